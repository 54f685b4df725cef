/*
 * photic.h -- C ABI of the GB300 implementation of photic's per-pixel
 * semi-analytical inversion (HOPE forward model + Nelder-Mead fit).
 *
 * All entry points are extern "C", take plain pointers and sizes, return an
 * int status (PHOTIC_OK == 0) and never exit the process.  Array arguments
 * named d_* are device pointers; the batch calls are asynchronous on the
 * given CUDA stream (pass NULL for the legacy default stream) and report
 * launch-time errors in their return value.  Errors raised while the
 * kernels run are read back with photic_sync().
 *
 * Mapping to the reference (file:line inside stblake/photic):
 *   photic_invert_batch        replaces the pixel loop of samodel()
 *                              model/samodel.c:901-1166 calling
 *                              samodel_optimise() model/samodel.c:1768
 *                              (cold start, no LUT, one region).
 *   photic_joint_invert_batch  the same loop with n_scenes = k per pixel,
 *                              the temporal joint fit
 *                              model/samodel.c:2463-2491, 2312-2353.
 *   photic_cost_batch          samodel_error() model/samodel.c:2432.
 *   photic_forward_batch       samodel_Rrs() model/samodel.c:2846.
 *   photic_interp_1d           interp_1d() model/common.c:298.
 *   photic_generate_scene      (new) synthetic scenes; no counterpart.
 * The link-compatible drop-ins samodel_Rrs / samodel_error /
 * samodel_optimise keep the reference signatures; they are declared in
 * photic_samodel.h together with the model_data layout they read.
 */
#ifndef PHOTIC_H
#define PHOTIC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHOTIC_MAX_BANDS 8
#define PHOTIC_MAX_SCENES 8
#define PHOTIC_MAX_HSTARTS 32

/* Return codes. */
enum {
  PHOTIC_OK = 0,
  PHOTIC_ERR_INVALID = 1,     /* bad argument or configuration */
  PHOTIC_ERR_CUDA = 2,        /* a CUDA call failed (message: photic_last_error) */
  PHOTIC_ERR_NOMEM = 3,       /* device allocation failed */
  PHOTIC_ERR_TIMEOUT = 4,     /* a bounded device wait gave up */
  PHOTIC_ERR_UNSUPPORTED = 5, /* configuration outside what the kernels implement */
  PHOTIC_ERR_IO = 6           /* a file is missing, unreadable or not in the expected format */
};

/* Arithmetic of the cost evaluations. */
enum {
  PHOTIC_PREC_FP64 = 0, /* IEEE double in the reference's operation order */
  PHOTIC_PREC_DF64 = 1, /* double-float (two FP32 words) on the FP32 pipes */
  PHOTIC_PREC_FP32 = 2, /* forward model in FP32 with the special-function
                           unit's exp and log; the simplex, its decisions, the
                           convergence and local-minimum tests and the final
                           re-evaluation in FP64 (not FP64-faithful) */
  PHOTIC_PREC_GUARDED = 3 /* FP64 decisions: every cost screened in
                             double-float, near ties re-evaluated in IEEE
                             double; same trajectory as PHOTIC_PREC_FP64 */
};

/* Per-pixel status word: low byte is the pixel state, bit 8 is set when
 * the kept start converged (nelmin ifault == 0), bits 16..23 hold the index
 * of the kept depth start. */
enum { PHOTIC_PX_FITTED = 0, PHOTIC_PX_MASKED = 1, PHOTIC_PX_INVALID = 2 };
#define PHOTIC_PX_CONVERGED 0x100
#define PHOTIC_PX_SERVED 0x200 /* photic_lut_invert_batch: outputs copied from a table entry */
#define PHOTIC_PX_HOT 0x400    /* photic_lut_invert_batch: fit hot-started from the previous pixel */

/* Parameter layouts of the temporal joint fit. */
enum {
  PHOTIC_LAYOUT_REFERENCE = 0, /* H, B, q shared; P, G, X per scene: n = 3 + 3k */
  PHOTIC_LAYOUT_SCENE_B = 1    /* H shared; B, P, G, X per scene:   n = 1 + 4k */
};

typedef struct photic_config {
  int32_t n_bands;                           /* bands per scene, 2..8 */
  double wavelengths[PHOTIC_MAX_BANDS];      /* nm, ascending */
  double theta_sun_deg;                      /* subsurface solar zenith (deg) */
  double theta_view_deg;                     /* subsurface view angle (deg) */
  double h_tide;                             /* tidal height added to depth */
  float nodata_value;                        /* masked-pixel marker */
  double reqmin;                             /* nelmin variance limit */
  int32_t konvge;                            /* iterations per convergence check */
  int32_t kcount;                            /* evaluation budget per nelmin call */
  int32_t n_hstarts;                         /* cold-start depths tried in order */
  double hstarts[PHOTIC_MAX_HSTARTS];
  double early_exit_per_scene;               /* keep a start when cost < this * scenes */
  int32_t precision;                         /* PHOTIC_PREC_* */
  int32_t layout;                            /* PHOTIC_LAYOUT_* (joint fit) */
  int32_t block_threads;                     /* launch shape; 0 = tuned default */
  int32_t blocks_per_sm;                     /* 0 = tuned default */
  double seed_step_scale;                    /* seeded starts: steps = this x the
                                                cold start's relative steps (1) */
} photic_config;

/* Outputs, structure of arrays.  Every pointer may be NULL (not written).
 * Single-scene calls write [npix]; the joint call writes per-pixel arrays
 * as [npix] and P/G/X as [n_obs] aligned with its inputs. */
typedef struct photic_outputs {
  float *depth;          /* H (m) */
  double *depth_f64;     /* H (m) in double precision */
  float *P, *G, *X;      /* 0.01 * |fitted parameter| */
  float *bottom_albedo;  /* sum_i q_i B_i */
  float *model_error;    /* cost at the kept optimum */
  float *rrs_error;      /* spectral RMS relative error (%) */
  float *K_min;          /* min over bands of K at the optimum */
  float *iod;            /* index of optical depth (%) */
  int32_t *evals;        /* cost evaluations over all starts */
  int32_t *evals_kept;   /* evaluations of the kept start */
  int32_t *status;       /* PHOTIC_PX_* | PHOTIC_PX_CONVERGED | start << 16 */
  double *params;        /* single-scene calls: [npix * 6] kept parameter vector
                            (H, 100B, q, 100P, 100G, 100X) as nelmin returned it */
  float *bottom_percent; /* photic_region_fit_batch: [npix * 3] share (%) of sand,
                            seagrass and coral in the pixel's own region */
  float *bottom_type;    /* photic_region_fit_batch: 1 + index of the largest share */
} photic_outputs;

/* Defaults: OLI-like bands 443/482/561/655 nm, sun 35 deg, nadir, the
 * reference's 8 cold depth starts (model/samodel.c:2216-2218), early exit
 * 2.5 per scene (:2404), reqmin 1e-10, konvge 100, kcount 2000, FP64. */
void photic_config_default(photic_config *cfg);

/* Validate cfg; PHOTIC_OK or PHOTIC_ERR_INVALID with a message. */
int photic_config_check(const photic_config *cfg);

/* Plain-method inversion of npix single-scene pixels.  Band b of pixel p
 * is d_rrs[p * pixel_stride + b * band_stride] (float).  d_seeds is NULL
 * (cold start) or [npix * 6] doubles: a start vector
 * (H, 100B, q, 100P, 100G, 100X) per pixel, NaN in the first slot meaning
 * cold start for that pixel. */
int photic_invert_batch(const photic_config *cfg, const float *d_rrs, int64_t npix,
                        int64_t pixel_stride, int64_t band_stride, const double *d_seeds,
                        const photic_outputs *out, void *stream);

/* photic_invert_batch with the pixels taken from the work queue in the order
 * d_order gives (device int32 [npix], a permutation of 0..npix-1; NULL: in
 * index order).  Results are written at each pixel's own index.  Taking the
 * fits expected to be longest first (e.g. the cold-start fallbacks of a
 * seeded batch) shortens the kernel's tail.  Not in guarded precision. */
int photic_invert_batch_ordered(const photic_config *cfg, const float *d_rrs, int64_t npix,
                                int64_t pixel_stride, int64_t band_stride,
                                const double *d_seeds, const int32_t *d_order,
                                const photic_outputs *out, void *stream);

/* Size of the static scratch array behind photic_invert_batch_noalloc. */
#define PHOTIC_NOALLOC_SCRATCH_BYTES 256

/* photic_invert_batch for callers that cannot allocate device memory.  No
 * counterpart in the reference.  Callers such as a serving process that
 * hands all of HBM to its own pool allocator at start-up, or a host
 * application that forbids allocation once its pipeline is running
 * (cudaMalloc can block on the device and breaks its memory accounting),
 * need an inversion that takes only the inputs and outputs they pass in.
 * This call allocates nothing: its 16 bytes of scratch (work-queue head and
 * error word) live in a static device array of PHOTIC_NOALLOC_SCRATCH_BYTES
 * that every GPU loading the library holds until the process exits.  The
 * first call on a device looks up that array's address (and lets CUDA load
 * the library's kernels), so make it before any stream capture.  All calls
 * share the one array and each clears it before its launch, so calls whose
 * kernels overlap on the GPU (two streams at once) race: serialise them.
 * Kernel-detected errors show only in the per-pixel status
 * (PHOTIC_PX_INVALID), so out->status must not be NULL (PHOTIC_ERR_INVALID
 * otherwise); photic_sync() does not see them.  Precisions PHOTIC_PREC_FP64
 * and PHOTIC_PREC_DF64 only: PHOTIC_PREC_GUARDED (whose request ring needs
 * its own scratch) and PHOTIC_PREC_FP32 return PHOTIC_ERR_UNSUPPORTED.
 * Otherwise arguments and results are those of photic_invert_batch. */
int photic_invert_batch_noalloc(const photic_config *cfg, const float *d_rrs, int64_t npix,
                                int64_t pixel_stride, int64_t band_stride,
                                const double *d_seeds, const photic_outputs *out,
                                void *stream);

/* Temporal joint fit: pixel p owns observations d_offsets[p] ..
 * d_offsets[p+1]-1 (CSR, int32, device); observation o has spectrum
 * d_rrs[o * n_bands .. +n_bands) and subsurface sun zenith
 * d_theta_sun_deg[o].  k = d_offsets[p+1]-d_offsets[p] must be 1..8. */
int photic_joint_invert_batch(const photic_config *cfg, const int32_t *d_offsets,
                              const double *d_theta_sun_deg, const float *d_rrs, int64_t npix,
                              int64_t n_obs, const photic_outputs *out, void *stream);

/* Cost of n parameter vectors (6 doubles each) against spectra
 * [n * n_bands] floats: samodel_error at one region. d_cost [n] doubles;
 * d_rrs_modelled [n * n_bands] doubles (NULL to skip). */
int photic_cost_batch(const photic_config *cfg, const float *d_rrs, const double *d_params,
                      int64_t n, double *d_cost, double *d_rrs_modelled, void *stream);

/* Spatially coherent synthetic scene of nrows x ncols pixels (the workload
 * of the lookup-table loop): one water mass (P, G, X within +/-10 % of
 * values drawn once from the seed), depth a smooth field over 0.5-25 m, the
 * bottom in three albedo classes with texture, N(0, noise_sigma) noise and
 * mask_frac of the pixels masked.  Writes rows row0 .. row0+n_rows-1:
 * [n_rows * ncols * n_bands] floats and, if d_truth != NULL,
 * [n_rows * ncols * 5] doubles (H, P, G, X, B). */
int photic_generate_field(const photic_config *cfg, uint64_t seed, int64_t nrows, int64_t ncols,
                          int64_t row0, int64_t n_rows, double mask_frac, double noise_sigma,
                          float *d_rrs, double *d_truth, void *stream);

/* Synthetic scene of the plain-method workload (photic_aux.cu):
 * writes [npix * n_bands] floats and, if d_truth != NULL, [npix * 5]
 * doubles (H, P, G, X, B). Pixels pix0 .. pix0+npix-1 of the scene. */
int photic_generate_scene(const photic_config *cfg, uint64_t seed, int64_t pix0, int64_t npix,
                          double mask_frac, double noise_sigma, float *d_rrs, double *d_truth,
                          void *stream);

/* Joint-fit synthetic stack: d_counts [npix] int32 scene counts in
 * [kmin, kmax]; after the caller forms offsets (exclusive scan),
 * photic_generate_joint fills theta_sun [n_obs], rrs [n_obs * n_bands] and
 * truth [n_obs * 5] (H shared per pixel). */
int photic_joint_counts(uint64_t seed, int64_t npix, int32_t kmin, int32_t kmax,
                        int32_t *d_counts, void *stream);
int photic_generate_joint(const photic_config *cfg, uint64_t seed, int64_t npix,
                          const int32_t *d_offsets, double theta_sun_min, double theta_sun_max,
                          double mask_frac, double noise_sigma, double *d_theta_sun,
                          float *d_rrs, double *d_truth, void *stream);

/* interp_1d of the reference (host function, no GPU needed). */
double photic_interp_1d(const double *X, const double *Y, int32_t n, double x);

/* Band constants of a configuration (host function): out[b*8 + 0..7] =
 * a0, a1, a_w, b_bw, sand reflectance, sec(theta_sun), sec(theta_view),
 * a_w(640). */
int photic_band_constants(const photic_config *cfg, double *out);

/* The reference's bottom reflectance table (model/samodel.c:236-287, in the
 * order of :464-475: sand, seagrass, coral, macrophytes, dark sediment,
 * coral sand, green algae, red algae) at cfg's bands (host function):
 * out[k * n_bands + b] for the first n_types (1..8) types, interpolated as
 * samodel() does (:550-618). */
int photic_bottom_reflectances(const photic_config *cfg, int32_t n_types, double *out);

/* Spatial-region fit (model/samodel.c:2957-3027 with n_spatial = 2): every
 * pixel of the [nrows][ncols][n_bands] grid (device, float) is fitted with
 * its 3 x 3 neighbourhood -- indexes clamped at the edges, neighbours with a
 * nodata band left out, the centre's slot the origin -- one depth, albedo and
 * q per region, shared P, G, X, and the cost's depth- and bottom-continuity
 * terms; depth is the origin-weighted mean (model/samodel.c:1999-2017).
 * Outputs per pixel; status carries the region count in bits 24-27.  One
 * scene, one bottom type, n_spatial = 2 only (photic_region_fit_batch with
 * n_bottoms = 1). */
int photic_region_invert_batch(const photic_config *cfg, const float *d_grid, int32_t nrows,
                               int32_t ncols, int32_t n_spatial, const photic_outputs *out,
                               void *stream);

/* The general fit of the reference's samodel() pixel loop
 * (model/samodel.c:901-1166 over samodel_optimise, :1768-2115).  d_grid
 * (device, float) is [n_scenes][nrows][ncols][n_bands]: n_scenes scenes of
 * the same place and bands, scene s with subsurface sun zenith
 * theta_sun_deg[s] (host array; NULL: cfg->theta_sun_deg for all).  Every
 * pixel is fitted alone (n_spatial = 1) or with its 3 x 3 neighbourhood
 * (n_spatial = 2, as photic_region_invert_batch), with n_bottoms = 1..3
 * bottom types (sand, seagrass, coral) mixed in every region: per region a
 * depth and per type an albedo and a mixing weight q, per scene P, G, X;
 * n = R + 2 n_bottoms R + 3 n_scenes unknowns (at most 96).  The
 * reference's default call is n_spatial = 2, n_bottoms = 3
 * (model/common.c:152).  d_h_empirical (NULL, or device [npix] doubles, NaN
 * for none) gives empirical depths: such a pixel takes that single depth
 * start, and one deeper than 8 m is fitted with sand alone
 * (model/samodel.c:1781, 1826-1830, 2208-2231).  Outputs per pixel, with P,
 * G, X as [npix][n_scenes], bottom_percent and bottom_type; status carries
 * the region count in bits 24-27.  Up to 128 regions x scenes x bands. */
int photic_region_fit_batch(const photic_config *cfg, const float *d_grid, int32_t n_scenes,
                            const double *theta_sun_deg, int32_t nrows, int32_t ncols,
                            int32_t n_spatial, int32_t n_bottoms, const double *d_h_empirical,
                            const photic_outputs *out, void *stream);

/* samodel()'s pixel loop with its dynamic lookup table, one scene, one
 * region, one bottom type (LUT 1, model/samodel.c:97, 649-660, 701-773,
 * 901-1215).  The shallow pixels of d_rrs (device, [npix][n_bands] float)
 * are sorted by the spectral index |(Rrs_1, Rrs_2, Rrs_3)| -- times the
 * spectral angle to rrs_noise[1..3] when use_noise and every band of
 * rrs_noise is at least 1e-6 (:590-600, 749-767) -- and the sorted list is
 * cut into n_chains contiguous slices (0: eight per resident lane, see
 * photic_lut_default_chains).  Each
 * slice runs the reference's loop as one of its threads does: a pixel whose
 * spectrum matches a stored fit within the match threshold (entries within
 * 10 % of the previous pixel's depth and K_min, model_spectral_diff_mean
 * :2792-2842) takes that fit's outputs (status PHOTIC_PX_SERVED, model_error
 * = the spectral difference, evals 0); any other pixel is fitted with cfg's
 * tolerances (the reference's are reqmin 1e-2, konvge 100, kcount 5000),
 * hot-started from the previous pixel when the last two were continuous
 * (PHOTIC_PX_HOT), and stored in the slice's table of n_lut slots (the
 * reference: 16000) when its model error is below the entry threshold and
 * its depth below 32 m; both thresholds adapt every 0.1 % of the slice.
 * d_empirical (NULL, or device [npix] floats, empirical_nodata for none)
 * is the reference's empirical depth grid (:702-710, 955-979): the pixels
 * are then ordered by it, and a pixel with one starts its fit there (hot or
 * cold, one start, depth = 1 m above -1 m, else |value|), a pixel without
 * one is fitted cold.
 * Optional device outputs: d_source [npix] (-2 masked, -1 fitted, else the
 * pixel whose fit served it), d_order [npix] (the sorted shallow pixels,
 * first *n_shallow entries), d_chain_stats [n_chains][4] (served, fitted,
 * final match and entry thresholds).  Host outputs: *n_shallow and
 * *n_chains_used (either may be NULL).  One slice is the reference on one
 * thread.  FP64 only (cfg->precision other than PHOTIC_PREC_FP64 returns
 * PHOTIC_ERR_UNSUPPORTED). */
typedef struct photic_lut_config {
  int32_t n_lut;                        /* slots per slice (the reference: 16000) */
  int64_t n_chains;                     /* slices; 0: eight per resident lane */
  int32_t use_noise;                    /* order by the spectral angle to rrs_noise */
  double rrs_noise[PHOTIC_MAX_BANDS];   /* the scene's noise spectrum (R_sigma) */
} photic_lut_config;

void photic_lut_config_default(photic_lut_config *lut);

/* The slice count n_chains = 0 stands for: eight per lane the kernel keeps
 * resident on this device (0 on error).  A slice is sequential; lanes that
 * finish theirs take the next from a queue, so several per lane keep the
 * kernel's tail to one short slice. */
int64_t photic_lut_default_chains(const photic_config *cfg);

int photic_lut_invert_batch(const photic_config *cfg, const photic_lut_config *lut,
                            const float *d_rrs, int64_t npix, const float *d_empirical,
                            float empirical_nodata, const photic_outputs *out,
                            int64_t *d_source, int64_t *d_order, double *d_chain_stats,
                            int64_t *n_shallow, int64_t *n_chains_used, void *stream);

/* samodel()'s pixel loop with its dynamic lookup table in the general
 * configuration: the fit of photic_region_fit_batch (3 x 3 regions,
 * mixtures of n_bottoms bottom types, stacks of n_scenes scenes) inside the
 * loop of photic_lut_invert_batch (model/samodel.c:649-1352).  d_grid
 * (device, float) is [n_scenes][nrows][ncols][n_bands]; theta_sun_deg as
 * for photic_region_fit_batch.  The shallow pixels (no band of any scene
 * nodata or negative) are sorted by |(sum over scenes of Rrs_1, Rrs_2,
 * Rrs_3)| -- times the spectral angle to the noise summed over the scenes
 * when rrs_noise (host, [n_scenes][n_bands]) is given, n_bands >= 4 and
 * every value is at least 1e-6 -- or by d_empirical (device [nrows *
 * ncols] floats, empirical_nodata for none).  Each slice of the sorted list
 * (lut->n_chains of them; 0: eight per resident warp, see
 * photic_region_lut_default_chains) runs the reference's loop on one warp:
 * a pixel whose table holds an entry with the same region count, within
 * 10 % of the previous pixel's depth and K_min, whose modelled Rrs of bands
 * 1..3 (averaged over scenes and regions where both are non-zero) differ
 * from the measured by at most the match threshold takes that fit's
 * outputs (PHOTIC_PX_SERVED, model_error = the difference, evals 0); any
 * other pixel is fitted -- hot-started from the previous pixel when the
 * last two were continuous (PHOTIC_PX_HOT: every region's depth at the
 * previous depth or the empirical one, each scene's P, G, X from the
 * previous fit) -- and entered into the table below the entry threshold
 * and 32 m.  A pixel with an empirical depth starts there; the depth that
 * selects sand alone above 8 m is the latest pixel's empirical depth in the
 * slice (0 before the first).  Outputs, d_source, d_order, d_chain_stats,
 * *n_shallow and *n_chains_used as for photic_lut_invert_batch, in the
 * layout of photic_region_fit_batch.  FP64 only. */
int photic_region_lut_invert_batch(const photic_config *cfg, const photic_lut_config *lut,
                                   const float *d_grid, int32_t n_scenes,
                                   const double *theta_sun_deg, int32_t nrows, int32_t ncols,
                                   int32_t n_spatial, int32_t n_bottoms, const double *rrs_noise,
                                   const float *d_empirical, float empirical_nodata,
                                   const photic_outputs *out, int64_t *d_source,
                                   int64_t *d_order, double *d_chain_stats, int64_t *n_shallow,
                                   int64_t *n_chains_used, void *stream);

/* Default slices of photic_region_lut_invert_batch for a configuration:
 * eight per warp of the general fit's kernel resident on this device (0 on
 * error or an unsupported configuration). */
int64_t photic_region_lut_default_chains(const photic_config *cfg, int32_t n_scenes,
                                         int32_t n_spatial, int32_t n_bottoms);

/* Depth uncertainty, the reference's ad hoc estimate (model/samodel.c:
 * 1368-1479): for each 0.25 m interval up to the deepest fitted depth (whole
 * metres, at most 30 m), n_samples pixels of the interval are drawn (up to
 * sqrt(npix) uniform probes each), every band moved by n * r_sigma[b] with
 * one n uniform in [-1, 1] per sample, and refitted with cfg; the interval's
 * sigma is the population standard deviation of the non-zero refitted
 * depths, and every pixel gets the sigma of the interval (d, d + 0.25]
 * holding its depth (0 elsewhere).  d_depth: [npix] fitted depths, positive,
 * 0 where not fitted; r_sigma: host [n_bands].  Draws come from Philox keyed
 * by seed (reproducible) instead of rand(); the refits are independent cold
 * starts instead of the reference's chain of hot starts.  Optional outputs:
 * d_table [120] sigmas, d_sample_pixel [120 * n_samples] (-1 = none found),
 * d_sample_depth [120 * n_samples]. */
int photic_depth_sigma(const photic_config *cfg, const float *d_rrs, int64_t npix,
                       const float *d_depth, const double *r_sigma, int32_t n_samples,
                       uint64_t seed, float *d_depth_sigma, double *d_table,
                       int32_t *d_sample_pixel, double *d_sample_depth, void *stream);

/* The same estimate for the general fit (model/samodel.c:1368-1479 as
 * samodel() runs it with regions, bottom mixtures or scene stacks): the
 * samples are drawn as photic_depth_sigma draws them, each sampled pixel's
 * regions (extract_Rrs_data) of every scene of d_grid ([n_scenes][nrows]
 * [ncols][n_bands], device) have every band moved by n * r_sigma[scene]
 * [band] (host, [n_scenes][n_bands]) and are refitted by the general fit
 * (photic_region_fit_batch's; cold depth starts, every bottom type: the
 * reference's h_empirical of 5 m, :1448).  Outputs as photic_depth_sigma. */
int photic_region_depth_sigma(const photic_config *cfg, const float *d_grid, int32_t n_scenes,
                              const double *theta_sun_deg, int32_t nrows, int32_t ncols,
                              int32_t n_spatial, int32_t n_bottoms, const float *d_depth,
                              const double *r_sigma, int32_t n_samples, uint64_t seed,
                              float *d_depth_sigma, double *d_table, int32_t *d_sample_pixel,
                              double *d_sample_depth, void *stream);

/* Launch-shape autotuner (new; no reference counterpart).  Times the
 * inversion (kind PHOTIC_TUNE_INVERT: block_threads 64/128/256 x blocks per
 * SM 0 (occupancy limit)/2/3/4) or the temporal joint fit (PHOTIC_TUNE_JOINT:
 * blocks per SM 2/3/4/6/8) on a seeded synthetic sample of sample_npix
 * pixels of cfg's workload, each candidate once untimed and once timed with
 * CUDA events, and writes the fastest into cfg->block_threads and
 * cfg->blocks_per_sm.  results (optional, max_results rows of 3 doubles)
 * receives (block_threads, blocks_per_sm, ms) per candidate.  Fits are
 * independent of the launch shape, so any choice gives the same outputs.
 * Synchronous on the legacy default stream. */
enum { PHOTIC_TUNE_INVERT = 0, PHOTIC_TUNE_JOINT = 1 };
int photic_autotune(photic_config *cfg, int32_t kind, int64_t sample_npix, double *results,
                    int32_t max_results, int32_t *n_results);

/* Waits for the stream, then reports any error recorded by the device
 * (bounded-wait timeouts, invalid inputs) since the previous call. */
int photic_sync(void *stream);

/* Measured pipe throughput of the current device, for roofline
 * denominators of the compute-bound kernels: FP64 and FP32 FMA (TFLOP/s,
 * 2 flops per FMA) and MUFU ex2 (T ops/s).  Synchronous; ~0.1 s. */
int photic_measure_peaks(double *fp64_tflops, double *fp32_tflops, double *mufu_tops);

/* BF16 GEMM on the tcgen05 tensor cores (FP32 accumulation in tensor
 * memory): C[M x N] = A[M x K] * B[N x K]^T, A and B row-major BF16 with
 * K contiguous (lda, ldb elements, multiples of 8; 16-byte aligned), C
 * row-major FP32.  K must be a positive multiple of 16.  The building block
 * of the surrogate network's training and inference (no counterpart in the
 * reference). */
int photic_gemm_bf16(const void *d_A, int32_t lda, const void *d_B, int32_t ldb, float *d_C,
                     int32_t ldc, int32_t M, int32_t N, int32_t K, void *stream);
/* The same with explicit core-matrix strides of the shared-memory operand
 * layout (lbo: between core matrices along K, sbo: along M/N; bytes);
 * photic_gemm_bf16 uses 128 / 1024.  For layout diagnostics.  Both must be
 * positive multiples of 16 with 768 + 15 * sbo + lbo + 128 <= 16384, so
 * that every core matrix the tensor core reads lies in the staged 128 x 64
 * tile; anything else returns PHOTIC_ERR_INVALID before any launch. */
int photic_gemm_bf16_strides(const void *d_A, int32_t lda, const void *d_B, int32_t ldb,
                             float *d_C, int32_t ldc, int32_t M, int32_t N, int32_t K,
                             int32_t lbo, int32_t sbo, void *stream);

/* ---- Learned warm start (no counterpart in the reference) --------------
 * An MLP 6 -> 128 -> 128 -> 128 -> 5 with SiLU maps the observed Rrs of the
 * four bands and the subsurface sun / view zenith (degrees) to
 * (ln P, ln G, ln X, B, H).  BF16 weights and activations, FP32
 * accumulation, trained and run on the tcgen05 tensor cores.  Features are
 * [R][6] floats, targets and predictions [R][5] floats. */
typedef struct photic_surrogate photic_surrogate;
int photic_surrogate_create(photic_surrogate **out, uint64_t seed);
int photic_surrogate_destroy(photic_surrogate *s);
int32_t photic_surrogate_num_params(void);
/* Copy the FP32 master parameters out (write = 0) or in (write = 1). */
int photic_surrogate_params(photic_surrogate *s, float *h_params, int32_t n, int32_t write);
/* Gradient of the mean squared error on standardised targets (no update);
 * d_grad [num_params]; d_loss (device float) is incremented by the loss. */
int photic_surrogate_grads(photic_surrogate *s, const float *d_x, const float *d_t, int32_t R,
                           float *d_grad, float *d_loss, void *stream);
/* One Adam step (lr) on a batch of R rows. */
int photic_surrogate_train_step(photic_surrogate *s, const float *d_x, const float *d_t,
                                int32_t R, float lr, float *d_loss, void *stream);
int photic_surrogate_infer(photic_surrogate *s, const float *d_x, int64_t R, float *d_y,
                           void *stream);
/* Start vectors for photic_invert_batch's d_seeds from the surrogate: pixels
 * whose predicted parameters reproduce the measured spectrum to an RMS of
 * resid_max or better get (H, 100B, 1, 100P, 100G, 100X); the others get NaN
 * (cold start).  d_resid (optional, [npix] float) receives the RMS. */
int photic_surrogate_seed(photic_surrogate *s, const photic_config *cfg, const float *d_rrs,
                          int64_t npix, double resid_max, double *d_seeds, float *d_resid,
                          void *stream);
/* As photic_surrogate_seed, with polish_iters (0..100) Levenberg-Marquardt
 * steps on each prediction before the residual test: single-precision
 * forward model, misfit in units of the noise sigma (resid_max / 3) plus a
 * weak pull towards the prediction, which picks the nearest point of the
 * underdetermined solution set.  The polished vector only seeds nelmin. */
int photic_surrogate_seed_polished(photic_surrogate *s, const photic_config *cfg,
                                   const float *d_rrs, int64_t npix, double resid_max,
                                   int32_t polish_iters, double *d_seeds, float *d_resid,
                                   void *stream);

/* The same Levenberg-Marquardt polish and residual test as
 * photic_surrogate_seed_polished, started without the network from the
 * reference's own cold-start guess (B = 4 Rrs(490), P = 0.072
 * (Rrs(490)/Rrs(550))^-1.7, G = 1.5 P, X = 30 a_w(640) Rrs(640);
 * model/samodel.c:2266-2273, 2342-2351) at depth h_guess (m; the polish
 * also tries 0.4 and 2.5 times it).  The baseline that shows what the
 * trained network adds to the polish; no counterpart in the reference. */
int photic_seed_polished_heuristic(const photic_config *cfg, const float *d_rrs, int64_t npix,
                                   double h_guess, double resid_max, int32_t polish_iters,
                                   double *d_seeds, float *d_resid, void *stream);

/* Instrumentation: if d_counter (device, unsigned long long) is not NULL,
 * later PHOTIC_PREC_GUARDED inversions add the number of exact FP64
 * re-evaluations they served to it.  Pass NULL to stop. */
int photic_set_counter(unsigned long long *d_counter);

/* Instrumentation of PHOTIC_PREC_GUARDED: if d_stats (device, 5 unsigned
 * long long) is not NULL, later guarded inversions add to it the number of
 * Nelder-Mead decisions taken on exact FP64 values already known, on the
 * double-float screen, and deferred to an exact FP64 evaluation, then the
 * lane-trips of the kernel's loop spent waiting for an exact value and
 * the lane-trips spent on a pixel.  Pass NULL to stop. */
int photic_set_guard_stats(unsigned long long *d_stats);

/* Message of the most recent error on this host thread. */
const char *photic_last_error(void);

/* Library version string. */
const char *photic_version(void);

#ifdef __cplusplus
}
#endif
#endif
