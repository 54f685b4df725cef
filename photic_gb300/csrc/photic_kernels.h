// photic_kernels.h -- launch arguments and launchers of the device code
// (internal to the library; the public ABI is include/photic.h).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/photic.h"
#include "photic_params.h"

namespace photic {

// Device error bits accumulated in the per-call error word.
enum : unsigned {
  PHOTIC_DEVERR_EVAL_CAP = 1u,     // a pixel exceeded the defensive evaluation cap
  PHOTIC_DEVERR_BAD_SCENES = 2u,   // a joint pixel had a scene count outside 1..8
  PHOTIC_DEVERR_MMA_TIMEOUT = 4u   // a tensor-core wait gave up
};

struct InvertArgs {
  FitParams fp;
  SceneConsts sc;
  DfScene ds;
  const float *rrs;
  int64_t npix, pixel_stride, band_stride;
  int32_t vec4;  // rrs is [npix][4], 16-byte aligned
  const double *seeds;
  photic_outputs out;
  unsigned long long *queue;
  unsigned int *error;
  unsigned long long *counters;  // optional: exact evaluations served (guarded)
  unsigned long long *guard_stats;  // optional [5] (guarded): decisions taken on exact
                                    // values, on the double-float screen, deferred to FP64;
                                    // lane trips waiting for an exact value, lane trips busy
  double early_exit;  // early-exit cost threshold (per-scene value * scenes)
  int32_t no_mask;    // fit every pixel: samodel_optimise has no mask test
  const int32_t *order;  // optional queue position -> pixel (e.g. long fits first)
};

size_t invert_smem_bytes(int block, int nb);
cudaError_t launch_invert(const InvertArgs &a, int precision, int block, int grid,
                          cudaStream_t s);
// Resident blocks per SM of the kernel that launch_invert would use (0 on error).
int invert_blocks_per_sm(const InvertArgs &a, int precision, int block);

// FP64-faithful inversion with double-float screening (photic_guarded.cu).
cudaError_t launch_guarded(const InvertArgs &a, int block, int grid, cudaStream_t s);
int guarded_blocks_per_sm(const InvertArgs &a, int block);

// samodel()'s pixel loop with the dynamic lookup table (photic_lut.cu).
struct LutKeyArgs {
  const float *rrs;  // [n_scenes][npix][n_bands]
  int64_t npix;
  int32_t n_bands;
  int32_t n_scenes;    // the keys sum blue, green and red over the scenes
  int32_t general;     // masked outputs in the region fit's layout (P, G, X per scene)
  float nodata;
  int32_t use_noise;   // order by index x spectral angle to noise[] (blue, green, red,
  double noise[3];     // each summed over the scenes)
  const float *emp;    // optional [npix] empirical depths: the key itself
  photic_outputs out;  // masked pixels' outputs are written here
  int64_t *source;     // optional [npix]: -2 for masked pixels
  float *keys;         // scratch [npix]
  uint8_t *flags;      // scratch [npix]
  int64_t *idx;        // scratch [npix]
};
struct LutArgs {
  InvertArgs inv;         // fp, sc, rrs ([npix][n_bands]), out, error, early_exit
  const int64_t *order;   // [n_shallow] sorted shallow pixels
  int64_t n_shallow, n_chains, cap;  // cap = table slots per chain
  double *ring;           // [n_chains][8][cap]
  int64_t *ring_src;      // [n_chains][cap]
  int64_t *source;        // optional [npix]: -1 fitted, else the pixel that served it
  double *chain_stats;    // optional [n_chains][4]: served, fitted, match, entry
  unsigned long long *queue;  // chain counter
  const float *emp;       // optional [npix] empirical depths, emp_nodata for none
  float emp_nodata;
};
cudaError_t lut_order(LutKeyArgs ka, int64_t *order, int64_t *n_shallow, cudaStream_t s);
cudaError_t launch_lut(const LutArgs &a, int grid, cudaStream_t s);
int lut_blocks_per_sm(const LutArgs &a);
int lut_block();

struct GenArgs {
  FitParams fp;
  SceneConsts sc;
  uint64_t seed;
  int64_t pix0, npix;
  double mask_frac, noise_sigma;
  float *rrs;
  double *truth;
  int64_t field_rows, field_cols;  // > 0: the spatially coherent scene of that size
};
cudaError_t launch_generate(const GenArgs &a, cudaStream_t s);

struct CostArgs {
  FitParams fp;
  SceneConsts sc;
  DfScene ds;
  int32_t precision;
  const float *rrs;
  const double *params;
  int64_t n;
  double *cost;
  double *rrs_modelled;
  double *details;  // optional [n][5]: Rrs error, model error, albedo, K_min, IOD
};
cudaError_t launch_cost(const CostArgs &a, cudaStream_t s);

struct JointArgs {
  FitParams fp;
  SceneConsts sc;             // band constants; sun secant per observation
  const int32_t *offsets;     // [npix + 1] CSR over observations
  const double *theta_sun;    // [n_obs] subsurface sun zenith (deg)
  const float *rrs;           // [n_obs][n_bands]
  int64_t npix;
  int32_t *list;              // [npix] pixel ids binned by scene count
  int32_t *bin_start;         // [8]
  int32_t *bin_count;         // [8]
  unsigned long long *queues; // [8] work-queue heads
  photic_outputs out;
  unsigned int *error;
};
// Bins pixels by scene count and runs one persistent kernel per count.
// Streams and events for running the per-k joint kernels side by side.
struct JointFork {
  cudaStream_t side[8];
  cudaEvent_t fork;
  cudaEvent_t join[8];
};
// per_sm: blocks per SM of each per-k kernel (0: the kernel's occupancy
// limit for the lane-group kernels, 4 for the thread-per-pixel ones).
cudaError_t launch_joint(const JointArgs &a, int32_t *fill, int sms, int per_sm, cudaStream_t s,
                         const JointFork *f);
// One per-k lane-group kernel (photic_joint_group.cu), n_bands <= 4.
cudaError_t launch_joint_group(const JointArgs &a, int k, int per_sm, int sms, cudaStream_t s);

struct JointGenArgs {
  FitParams fp;
  SceneConsts sc;
  uint64_t seed;
  int64_t npix;
  const int32_t *offsets;
  double theta_min, theta_max, mask_frac, noise_sigma;
  double *theta_sun;
  float *rrs;
  double *truth;
};
cudaError_t launch_joint_counts(uint64_t seed, int64_t npix, int32_t kmin, int32_t kmax,
                                int32_t *counts, cudaStream_t s);
cudaError_t launch_generate_joint(const JointGenArgs &a, cudaStream_t s);

// BF16 TN GEMM on tcgen05 (photic_gemm.cu).
enum { EPI_F32 = 0, EPI_BIAS_F32 = 1, EPI_BIAS_SILU = 2, EPI_DSILU = 3 };
struct GemmArgs {
  const void *A;   // __nv_bfloat16 [M][lda]
  const void *B;   // __nv_bfloat16 [N][ldb]
  int lda, ldb, M, N, K;
  float *C;        // EPI_F32 / EPI_BIAS_F32 output [M][ldc]
  int ldc;
  void *O;         // __nv_bfloat16 output [M][ldo] (SILU / DSILU)
  int ldo;
  float *Z;        // pre-activation [M][ldz]: written by SILU, read by DSILU
  int ldz;
  const float *bias;
  unsigned int *error;
  int lbo, sbo;    // core-matrix strides of the shared-memory layout (bytes)
  int epi;
  int ksplit;      // > 1: split K over this many CTAs (EPI_F32 only) ...
  float *partial;  // ... with partial sums in [ksplit][M][N] scratch
};
cudaError_t launch_gemm(const GemmArgs &g, cudaStream_t s);

// Surrogate MLP (photic_mlp.cu): 6 (padded 16) -> 128 -> 128 -> 128 -> 5
// (padded 16).  FP32 master parameters, flat, in this order.
constexpr int kMlpIn = 16, kMlpH = 128, kMlpOut = 16;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kMlpH * kMlpIn;
constexpr int kOffW2 = kOffB1 + kMlpH;
constexpr int kOffB2 = kOffW2 + kMlpH * kMlpH;
constexpr int kOffW3 = kOffB2 + kMlpH;
constexpr int kOffB3 = kOffW3 + kMlpH * kMlpH;
constexpr int kOffW4 = kOffB3 + kMlpH;
constexpr int kOffB4 = kOffW4 + kMlpOut * kMlpH;
constexpr int kMlpParams = kOffB4 + kMlpOut;

struct MlpState {
  float *P, *M, *V;  // parameters and Adam moments
  __nv_bfloat16 *W1b, *W2b, *W3b, *W4b, *W2t, *W3t, *W4t;
  float *in_mean, *in_std, *out_mean, *out_std;  // [16] each
};
constexpr int kMlpSplitK = 64;  // K splits of the weight-gradient products
struct MlpWork {
  __nv_bfloat16 *X0, *A1, *A2, *A3, *dY, *dZ, *dZ2, *T1, *T2;
  float *Z1, *Z2, *Z3, *Y, *G4t, *grad;
  float *splitk;  // [kMlpSplitK][128][128] partial sums (training)
};
// Band constants in single precision, for the seed polish.
struct SceneF32 {
  float refl[8], aw[8], a0[8], a1[8], eS[8], bbw[8];
  float sec_sun, sec_view;
};

struct SeedArgs {
  FitParams fp;
  SceneConsts sc;
  SceneF32 sf;
  const float *rrs;
  const float *y;     // [npix][5] surrogate outputs (ln P, ln G, ln X, B, H)
  // y == nullptr: the guess is the reference's cold start of P, G, X and B
  // (model/samodel.c:2266-2273, 2342-2351) with depth h_guess
  double h_guess;
  int64_t npix;
  double resid_max;
  int32_t polish_iters;  // Levenberg-Marquardt steps on the seed (0: none)
  double *seeds;      // [npix][6]
  float *resid;       // optional [npix]
};
cudaError_t mlp_refresh(const MlpState &st, cudaStream_t s);
cudaError_t mlp_forward(const MlpState &st, const float *x, int R, int Rpad, MlpWork &w,
                        unsigned int *err, cudaStream_t s);
cudaError_t mlp_backward(const MlpState &st, const float *x, const float *t, int R, int Rpad,
                         MlpWork &w, float *loss, unsigned int *err, cudaStream_t s);
cudaError_t mlp_adam(const MlpState &st, const MlpWork &w, float lr, int step, cudaStream_t s);
cudaError_t mlp_denorm(const MlpState &st, const MlpWork &w, int R, float *y, cudaStream_t s);
cudaError_t mlp_features(const float *rrs, int64_t npix, int nb, float th_sun, float th_view,
                         float *x, cudaStream_t s);
cudaError_t mlp_seeds(const SeedArgs &a, cudaStream_t s);

struct ForwardArgs {
  FitParams fp;
  SceneConsts sc;
  const double *params;  // [n][7]: P, G, X, B, q, H, Delta
  const double *rrs440, *rrs490;
  int64_t n;
  double *rrs, *K;       // [n][n_bands]
  double *parts;         // optional [n][n_bands][4]: rho, rrs_dp, rrs_bottom, rrs
  // optional bottom mixture per row: [n][6] = B_0..B_2, q_0..q_2 (q already
  // normalised, as samodel_Rrs takes them) of n_bottoms types with
  // reflectances sc.refl_k; replaces the row's B and q
  const double *mix;
  int32_t n_bottoms;
};
cudaError_t launch_forward(const ForwardArgs &a, cudaStream_t s);

struct EmpSeedArgs {
  FitParams fp;
  SceneConsts sc;
  const float *rrs;      // [npix][n_bands]
  const double *h;       // [npix] empirical depth, NaN = none
  int64_t npix;
  double *seeds;         // [npix][6]
};
cudaError_t launch_empirical_seeds(const EmpSeedArgs &a, cudaStream_t s);

// Spatial-region fit, 3 x 3 neighbourhoods (photic_region.cu).
// The general single-scene fit (photic_region.cu): pixels alone or with
// their 3 x 3 neighbourhood, 1..3 bottom types mixed per region.
constexpr int kRegionMaxR = 9;        // regions of a 3 x 3 neighbourhood
constexpr int kRegionMaxParams = 66;  // 9 + 2 * 3 * 9 + 3 (one scene)
struct RegionArgs {
  FitParams fp;
  SceneConsts sc;
  const float *grid;            // grid mode: [nrows][ncols][n_bands]
  int nrows, ncols;
  int64_t npix;                 // problems (grid: nrows * ncols)
  int32_t n_scenes;             // scenes of the same bands; grid: [S][nrows][ncols][n_bands]
  double sec_sun[kMaxScenes];   // per-scene secant of the subsurface sun zenith
  int32_t n_spatial;            // 1: each pixel alone, 2: 3 x 3 regions
  int32_t n_bottoms;            // bottom types 1..3 (sand, seagrass, coral)
  const double *h_emp;          // optional [npix] empirical depth (NaN: none)
  int32_t no_mask;              // skip the pixel loop's mask test (list mode)
  // list mode (the per-pixel drop-ins): problem p has list_R[p] regions with
  // spectra list_rrs[((p * 9 + r) * n_scenes + s) * n_bands + b] and origin
  // list_origin[p]
  const float *list_rrs;
  const int32_t *list_R, *list_origin;
  // optional [npix][eval_stride] in: parameters to evaluate instead of
  // fitting (samodel_error); out: the kept parameter vector of a fit
  const double *eval_params;
  double *list_params;
  int32_t eval_stride;
  double *eval_cost;            // [npix] cost at eval_params
  double *eval_rm;              // [npix][9][n_scenes][n_bands] modelled Rrs
  double *eval_det;             // [npix][8]: Rrs error, model error, albedo, the last
                                // scene's K_min (the cost's), IOD, K_min over all
                                // scenes (the post-fit product's)
  unsigned long long *queue;    // work-queue head (zeroed): pixels, or chains
  photic_outputs out;           // per pixel (P, G, X: [npix][n_scenes]); status carries
                                // the region count << 24
  unsigned int *error;
  // chain mode (samodel()'s pixel loop with its lookup table, grid mode):
  // the sorted shallow pixels cut into n_chains contiguous slices, one warp
  // per slice at a time
  const int64_t *order;         // [n_shallow]; NULL: every pixel from the queue
  int64_t n_shallow, n_chains, cap;  // cap: table slots per chain
  int32_t entry_stride;         // doubles per table entry
  double *ring;                 // [n_chains][cap][entry_stride]
  int64_t *ring_src;            // [n_chains][cap]: the pixel whose fit an entry holds
  int64_t *source;              // optional [npix]: -1 fitted, else the serving pixel
  double *chain_stats;          // optional [n_chains][4]: served, fitted, match, entry
  const float *emp;             // optional [npix] empirical depths (emp_nodata: none)
  float emp_nodata;
};
// Doubles of one table entry of the general loop: region count, depth,
// K_min, P, G, X per scene, modelled Rrs of bands 1..3 per region and scene.
constexpr int region_entry_stride(int n_scenes) { return 3 + 3 * n_scenes + 27 * n_scenes; }
// Parameters of a fit with up to max_regions regions, n_bottoms types and
// n_scenes scenes.
int region_max_params(int max_regions, int n_bottoms, int n_scenes);
// warps: when non-NULL, no launch -- the number of resident warps of the
// kernel that max_params selects is returned there.
cudaError_t launch_region(const RegionArgs &a, int max_params, int sms, int per_sm,
                          cudaStream_t s, int64_t *warps = nullptr);

// Depth uncertainty by re-inversion of perturbed samples (photic_aux.cu).
constexpr int kDsMaxIntervals = 120;  // 30 m in 0.25 m steps
struct DepthSigmaArgs {
  const float *rrs;          // [npix][n_bands] scene spectra
  const float *depth;        // [npix] fitted depths (positive, 0 = not fitted)
  int64_t npix;
  int n_bands, n_samples, n_trials;
  double interval;           // 0.25 m
  double r_sigma[8];         // deep-water sigma per band
  float nodata;
  uint64_t seed;
  unsigned int *max_bits;    // scratch: deepest depth (float bits), zeroed
  int32_t *sample_pixel;     // [kDsMaxIntervals * n_samples], -1 = none
  float *sample_rrs;         // optional [kDsMaxIntervals * n_samples][n_bands]
  float *sample_n;           // optional [kDsMaxIntervals * n_samples]: the draws n
  const double *sample_depth;  // refitted depths of the samples
  double *table;             // [kDsMaxIntervals]
  float *depth_sigma;        // [npix]
};
cudaError_t launch_depth_sigma_select(const DepthSigmaArgs &a, cudaStream_t s);
// The depth uncertainty's samples for the general fit: each sampled pixel's
// regions (extract_Rrs_data, model/samodel.c:2957-3027) with every band of
// every scene moved by n R_sigma[scene][band], as region lists.
struct RegionSampleArgs {
  const float *grid;           // [n_scenes][nrows][ncols][n_bands]
  int nrows, ncols, n_scenes, n_bands, n_spatial;
  float nodata;
  double r_sigma[kMaxScenes * 8];  // [scene][band]
  const int32_t *sample_pixel;  // [ns], -1 = none (no regions)
  const float *sample_n;        // [ns]
  int64_t ns;
  float *list_rrs;              // [ns][9][n_scenes][n_bands]
  int32_t *list_R, *list_origin;  // [ns]
};
cudaError_t launch_region_samples(const RegionSampleArgs &a, cudaStream_t s);
cudaError_t launch_depth_sigma_finish(const DepthSigmaArgs &a, cudaStream_t s);

// Throughput probes (TFLOP/s of FP64 and FP32 FMA, Tops/s of MUFU ex2).
cudaError_t measure_peaks(double *fp64_tflops, double *fp32_tflops, double *mufu_tops);

}  // namespace photic
