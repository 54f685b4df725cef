// photic_aux.cu -- synthetic scene generator and the batched cost kernel.
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_dfcost.cuh"
#include "photic_fp64.cuh"
#include "photic_kernels.h"

namespace photic {

namespace {

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): counter (idx, block,
// stream), key = 64-bit seed.  Same stream of uniforms as the CPU generator
// used by the tests.
__device__ __forceinline__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__device__ __forceinline__ void draw4(uint64_t seed, uint64_t idx, uint32_t block, uint32_t stream,
                                      double u[4]) {
  uint32_t c[4] = {(uint32_t)idx, (uint32_t)(idx >> 32), block, stream};
  philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
#pragma unroll
  for (int i = 0; i < 4; i++) u[i] = ((double)c[i] + 0.5) * 2.3283064365386963e-10;
}

__device__ __forceinline__ double log_uniform(double u, double lo, double hi) {
  return exp(log(lo) + u * (log(hi) - log(lo)));
}

// Self-consistent spectrum of truth (H, P, G, X, B): the forward model's Y
// exponent depends on the spectrum itself, so iterate spectrum -> model.
template <int NB>
__device__ void synthesise(const FitParams &fp, const SceneConsts &sc, double H, double P,
                           double G, double X, double B, double *rrs) {
  double x[6] = {H, 100.0 * B, 1.0, 100.0 * P, 100.0 * G, 100.0 * X};
  double cur[NB];
#pragma unroll
  for (int b = 0; b < NB; b++) cur[b] = 0.01;
  for (int it = 0; it < 30; it++) {
    PixelF64<NB> px;
    pixel_setup_f64<NB>(fp, sc, cur, px);
    CostDetailsF64 det;
    cost_f64<true, NB>(fp, sc, px, x, &det);
#pragma unroll
    for (int b = 0; b < NB; b++) cur[b] = det.Rm[b];
  }
#pragma unroll
  for (int b = 0; b < NB; b++) rrs[b] = cur[b];
}

// One smooth field over the scene in [0, 1]: three seeded harmonics.
__device__ double field_value(uint64_t seed, uint32_t which, double u, double v) {
  double s = 0.0, norm = 0.0;
  for (int h = 0; h < 3; h++) {
    double w[4];
    const double amp = 1.0 / (double)(1 << h);
    draw4(seed, (uint64_t)(which * 4u + (uint32_t)h), 7u, 1u, w);
    const double fx = 1.0 + floor(4.0 * w[0]), fy = 1.0 + floor(4.0 * w[1]);
    const double ph = 2.0 * kPi * w[2];
    s += amp * sin(2.0 * kPi * (fx * u + fy * v) + ph);
    norm += amp;
  }
  return 0.5 + 0.5 * s / norm;
}

template <int NB>
__global__ void generate_kernel(GenArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.npix) return;
  const int nb = a.fp.n_bands;
  const uint64_t p = (uint64_t)(a.pix0 + i);
  double u0[4], u1[4];
  draw4(a.seed, p, 0u, 0u, u0);
  draw4(a.seed, p, 1u, 0u, u1);
  double H, P, G, X, B;
  if (a.field_rows > 0) {
    // the spatially coherent scene: one water mass (P, G, X within +/-10 %
    // of values drawn once), depth a smooth field over 0.5-25 m, the bottom
    // in three albedo classes with +/-5 % texture
    const int64_t row = (int64_t)p / a.field_cols, col = (int64_t)p % a.field_cols;
    const double u = ((double)row + 0.5) / (double)a.field_rows;
    const double v = ((double)col + 0.5) / (double)a.field_cols;
    double w[4];
    draw4(a.seed, 0u, 9u, 1u, w);
    const double tH = field_value(a.seed, 0u, u, v), tB = field_value(a.seed, 4u, u, v);
    const double cls = tB < 0.4 ? 0.08 : (tB < 0.6 ? 0.2 : 0.4);
    H = 0.5 + 24.5 * tH * tH;
    P = log_uniform(w[0], 0.01, 0.05) * (0.9 + 0.2 * field_value(a.seed, 1u, u, v));
    G = log_uniform(w[1], 0.01, 0.08) * (0.9 + 0.2 * field_value(a.seed, 2u, u, v));
    X = log_uniform(w[2], 0.002, 0.02) * (0.9 + 0.2 * field_value(a.seed, 3u, u, v));
    B = cls * (0.95 + 0.1 * field_value(a.seed, 5u, u, v));
  } else {
    H = 0.5 + 24.5 * u0[0];
    P = log_uniform(u0[1], 0.005, 0.1);
    G = log_uniform(u0[2], 0.005, 0.2);
    X = log_uniform(u0[3], 0.001, 0.05);
    B = 0.05 + 0.45 * u1[0];
  }
  double r[NB];
  synthesise<NB>(a.fp, a.sc, H, P, G, X, B, r);
  for (int b = 0; b < nb; b += 2) {
    double u[4];
    draw4(a.seed, p, 2u + (uint32_t)(b / 4), 0u, u);
    const double rad = sqrt(-2.0 * log(u[b % 4]));
    const double ang = 2.0 * kPi * u[(b % 4) + 1];
    r[b] += a.noise_sigma * rad * cos(ang);
    if (b + 1 < nb) r[b + 1] += a.noise_sigma * rad * sin(ang);
  }
  float *o = a.rrs + i * nb;
  for (int b = 0; b < nb; b++) o[b] = (float)r[b];
  if (u1[1] < a.mask_frac) {
    if (u1[2] < 0.5) {
      for (int b = 0; b < nb; b++) o[b] = a.fp.nodata;
    } else {
      o[nb - 1] = -fabsf(o[nb - 1]) - 1.0e-3f;
    }
  }
  if (a.truth) {
    double *t = a.truth + i * 5;
    t[0] = H;
    t[1] = P;
    t[2] = G;
    t[3] = X;
    t[4] = B;
  }
}

__global__ void joint_counts_kernel(uint64_t seed, int64_t npix, int32_t kmin, int32_t kmax,
                                    int32_t *counts) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  double u[4];
  draw4(seed, (uint64_t)p, 0u, 1u, u);
  int k = kmin + (int)(u[0] * (double)(kmax - kmin + 1));
  if (k > kmax) k = kmax;
  counts[p] = k;
}

// Stack of k scenes over one pixel: shared depth, per-scene P, G, X, B and
// sun zenith U(theta_min, theta_max), independent noise.  The first
// observation carries the pixel's mask, as in the CPU generator.
template <int NB>
__global__ void generate_joint_kernel(const __grid_constant__ JointGenArgs a) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  const int nb = a.fp.n_bands;
  const int o0 = a.offsets[p], k = a.offsets[p + 1] - o0;
  double uH[4];
  draw4(a.seed, (uint64_t)p, 1u, 1u, uH);
  const double H = 0.5 + 24.5 * uH[0];
  for (int s = 0; s < k; s++) {
    const uint64_t obs = (uint64_t)(o0 + s);
    double u0[4], u1[4];
    draw4(a.seed, obs, 0u, 2u, u0);
    draw4(a.seed, obs, 1u, 2u, u1);
    const double P = log_uniform(u0[0], 0.005, 0.1);
    const double G = log_uniform(u0[1], 0.005, 0.2);
    const double X = log_uniform(u0[2], 0.001, 0.05);
    const double B = 0.05 + 0.45 * u0[3];
    const double th = a.theta_min + (a.theta_max - a.theta_min) * u1[0];
    a.theta_sun[obs] = th;
    SceneConsts sc = a.sc;
    double t = th;
    t *= 3.141592653589793 / 180.0;
    sc.sec_sun = 1.0 / cos(t);
    double r[NB];
    synthesise<NB>(a.fp, sc, H, P, G, X, B, r);
    for (int b = 0; b < nb; b += 2) {
      double u[4];
      draw4(a.seed, obs, 2u + (uint32_t)(b / 4), 2u, u);
      const double rad = sqrt(-2.0 * log(u[b % 4]));
      const double ang = 2.0 * kPi * u[(b % 4) + 1];
      r[b] += a.noise_sigma * rad * cos(ang);
      if (b + 1 < nb) r[b + 1] += a.noise_sigma * rad * sin(ang);
    }
    float *out = a.rrs + obs * nb;
    for (int b = 0; b < nb; b++) out[b] = (float)r[b];
    if (s == 0 && uH[1] < a.mask_frac) {
      if (uH[2] < 0.5) {
        for (int b = 0; b < nb; b++) out[b] = a.fp.nodata;
      } else {
        out[nb - 1] = -fabsf(out[nb - 1]) - 1.0e-3f;
      }
    }
    if (a.truth) {
      double *tr = a.truth + obs * 5;
      tr[0] = H;
      tr[1] = P;
      tr[2] = G;
      tr[3] = X;
      tr[4] = B;
    }
  }
}

// Forward model of n parameter sets (P, G, X, B, q, H, Delta per row, 7
// doubles) with caller-given Rrs(440)/Rrs(490).
__global__ void forward_kernel(const __grid_constant__ ForwardArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const double *x = a.params + i * 7;
  const double chi = a.rrs440[i] / a.rrs490[i];
  double Y = 3.44 * (1.0 - 3.17 * fm::exp_t(-2.01 * chi));
  if (Y < 0.0) Y = 0.0;
  if (Y > 2.5) Y = 2.5;
  const double qB = x[4] * x[3];
  for (int b = 0; b < a.fp.n_bands; b++) {
    double K, parts[4];
    double rho = qB * a.sc.refl[b];
    if (a.mix) {  // sum_i q_i B_i rho_i(lambda), model/samodel.c:2878-2883
      const double *m = a.mix + i * 6;
      rho = 0.0;
      for (int k = 0; k < a.n_bottoms; k++) rho += m[3 + k] * m[k] * a.sc.refl_k[k][b];
    }
    const double r = forward_band_rho_f64(a.sc, b, x[0], x[1], x[2], rho, x[5], x[6],
                                          pow(a.sc.ratio440[b], Y), &K, parts);
    a.rrs[i * a.fp.n_bands + b] = r;
    if (a.K) a.K[i * a.fp.n_bands + b] = K;
    if (a.parts)
      for (int j = 0; j < 4; j++) a.parts[(i * a.fp.n_bands + b) * 4 + j] = parts[j];
  }
}

// Start vectors of the reference's empirical-depth path (one start at the
// pixel's empirical depth, model/samodel.c:2208-2231): the cold start of
// model/samodel.c:2249-2353 with H replaced; NaN where no depth is given.
template <int NB>
__global__ void empirical_seeds_kernel(const __grid_constant__ EmpSeedArgs a) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  double *sd = a.seeds + p * 6;
  const double h = a.h[p];
  if (isnan(h)) {
    sd[0] = h;
    return;
  }
  const int nb = a.fp.n_bands;
  double r[NB];
#pragma unroll
  for (int b = 0; b < NB; b++) r[b] = b < nb ? (double)a.rrs[p * nb + b] : 0.0;
  PixelF64<NB> px;
  pixel_setup_f64<NB>(a.fp, a.sc, r, px);
  double start[6], step[6];
  cold_start_f64<NB>(a.fp, px, start, step);
  start[0] = h;
#pragma unroll
  for (int i = 0; i < 6; i++) sd[i] = start[i];
}

template <int NB>
__global__ void cost_kernel_df(const __grid_constant__ CostArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int nb = a.fp.n_bands;
  float r[NB];
#pragma unroll
  for (int b = 0; b < NB; b++) r[b] = b < nb ? a.rrs[i * nb + b] : 0.0f;
  PixelDF<NB> px;
  pixel_setup_df<NB>(a.fp, a.ds, r, px);
  df64 x[6];
#pragma unroll
  for (int k = 0; k < 6; k++) x[k] = df_from_double(a.params[i * 6 + k]);
  a.cost[i] = df_to_double(cost_df<false, NB>(a.fp, a.ds, px, x, nullptr));
}

template <int NB>
__global__ void cost_kernel(CostArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int nb = a.fp.n_bands;
  double r[NB];
#pragma unroll
  for (int b = 0; b < NB; b++) r[b] = b < nb ? (double)a.rrs[i * nb + b] : 0.0;
  PixelF64<NB> px;
  pixel_setup_f64<NB>(a.fp, a.sc, r, px);
  double x[6];
#pragma unroll
  for (int k = 0; k < 6; k++) x[k] = a.params[i * 6 + k];
  CostDetailsF64 det;
  const double c = cost_f64<true, NB>(a.fp, a.sc, px, x, &det);
  a.cost[i] = c;
  if (a.rrs_modelled)
    for (int b = 0; b < nb; b++) a.rrs_modelled[i * nb + b] = det.Rm[b];
  if (a.details) {
    double *d = a.details + i * 5;
    d[0] = det.rrs_error;
    d[1] = det.model_error;
    d[2] = det.bottom_albedo;
    d[3] = det.K_min;
    d[4] = det.iod;
  }
}

// ---- depth uncertainty (model/samodel.c:1368-1479) -------------------
// The reference's ad hoc depth error: for each 0.25 m depth interval up to
// the deepest fitted depth (whole metres, at most 30 m), refit 128 pixels
// drawn at random from that interval with every band moved by the same
// random multiple n in [-1, 1] of the scene's deep-water sigma, and give
// every pixel of the interval the standard deviation of the refitted depths.
// Draws come from Philox (seeded, reproducible) instead of rand().

__device__ __forceinline__ bool approx_f(float a, float b, float eps) {
  const float d = fabsf(a - b);
  return d <= (fabsf(a) < fabsf(b) ? fabsf(b) : fabsf(a)) * eps;
}

// Deepest fitted depth as float bits (non-negative floats order as ints).
__global__ void ds_max_kernel(const float *depth, int64_t npix, unsigned int *max_bits) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float v = 0.0f;
  if (p < npix) {
    v = depth[p];
    if (!(v > 0.0f) || approx_f(v, 0.0f, 1.0e-4f)) v = 0.0f;  // array_max2 skips 0
  }
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0 && v > 0.0f) atomicMax(max_bits, __float_as_uint(v));
}

__device__ __forceinline__ int ds_intervals(const unsigned int *max_bits, double interval) {
  const float mx = __uint_as_float(*max_bits);
  double m = interval * (double)((int)mx / interval);  // model/samodel.c:1384
  if (m > 30.0) m = 30.0;
  int n = (int)(m / interval);
  return n < kDsMaxIntervals ? n : kDsMaxIntervals;
}

// One thread per (interval, sample): find a pixel of the interval by up to
// n_trials uniform probes, draw n, write the perturbed spectrum (or a
// nodata spectrum when none was found).
__global__ void ds_select_kernel(const __grid_constant__ DepthSigmaArgs a) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (int64_t)kDsMaxIntervals * a.n_samples) return;
  const int k = (int)(g / a.n_samples);
  const int nb = a.n_bands;
  const int n_int = ds_intervals(a.max_bits, a.interval);
  const double d = k * a.interval;
  int64_t found = -1;
  if (k < n_int) {
    for (int t = 0; t < a.n_trials && found < 0; t++) {
      uint32_t c[4] = {(uint32_t)g, (uint32_t)(g >> 32), (uint32_t)t, 0xD5u};
      philox(c, (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
      const int64_t p = (int64_t)(((uint64_t)c[0] * (uint64_t)a.npix) >> 32);
      const float dp = a.depth[p];
      if (dp > d && dp < d + a.interval) found = p;
    }
  }
  a.sample_pixel[g] = (int32_t)found;
  float *out = a.sample_rrs ? a.sample_rrs + g * nb : nullptr;
  if (found < 0) {
    if (out)
      for (int b = 0; b < nb; b++) out[b] = a.nodata;
    if (a.sample_n) a.sample_n[g] = 0.0f;
    return;
  }
  uint32_t c[4] = {(uint32_t)g, (uint32_t)(g >> 32), 0xFFFFFFFFu, 0xD6u};
  philox(c, (uint32_t)a.seed, (uint32_t)(a.seed >> 32));
  const double u0 = ((double)c[0] + 0.5) * 2.3283064365386963e-10;
  const double u1 = ((double)c[1] + 0.5) * 2.3283064365386963e-10;
  const float n = u0 < 0.5 ? (float)u1 : -1.0f * (float)u1;  // frand2(1.0)
  if (a.sample_n) a.sample_n[g] = n;
  if (!out) return;
  for (int b = 0; b < nb; b++) {
    const float refl = a.rrs[found * nb + b];
    double v = (double)refl;
    if (!approx_f(n, 0.0f, 1.0e-6f)) v += (double)n * a.r_sigma[b];
    out[b] = (float)v;
  }
}

// One thread per interval: mean (rounded to float, as vec_mean2_double
// returns it) and population standard deviation of the non-zero refitted
// depths (model/common.c:877-940).
__global__ void ds_table_kernel(const __grid_constant__ DepthSigmaArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kDsMaxIntervals) return;
  const int n_int = ds_intervals(a.max_bits, a.interval);
  double sigma = 0.0;
  if (k < n_int) {
    const double *v = a.sample_depth + (int64_t)k * a.n_samples;
    double total = 0.0;
    int count = 0;
    for (int s = 0; s < a.n_samples; s++)
      if (!approx_f((float)v[s], 0.0f, 1.0e-4f)) {
        total += v[s];
        count++;
      }
    if (count > 0) {
      const double mean = (double)(float)(total / (double)count);
      double sumdev = 0.0;
      for (int s = 0; s < a.n_samples; s++)
        if (!approx_f((float)v[s], 0.0f, 1.0e-4f)) sumdev += pow(v[s] - mean, 2.0);
      sigma = sqrt(sumdev / (double)count);
    }
  }
  a.table[k] = sigma;
}

// Per pixel: the sigma of the interval (d, d + interval] holding its depth.
__global__ void ds_map_kernel(const __grid_constant__ DepthSigmaArgs a) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  const int n_int = ds_intervals(a.max_bits, a.interval);
  const float dp = a.depth[p];
  float s = 0.0f;
  if (dp > 0.0f) {
    double d = 0.0;
    for (int k = 0; k < n_int; k++, d += a.interval)
      if (dp > d && dp <= d + a.interval) {
        s = (float)a.table[k];
        break;
      }
  }
  a.depth_sigma[p] = s;
}

}  // namespace

cudaError_t launch_generate(const GenArgs &a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const int block = 128;
  const int64_t grid = (a.npix + block - 1) / block;
  if (a.fp.n_bands == 4) generate_kernel<4><<<(unsigned)grid, block, 0, s>>>(a);
  else generate_kernel<8><<<(unsigned)grid, block, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_joint_counts(uint64_t seed, int64_t npix, int32_t kmin, int32_t kmax,
                                int32_t *counts, cudaStream_t s) {
  if (npix <= 0) return cudaSuccess;
  joint_counts_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, s>>>(seed, npix, kmin, kmax,
                                                                      counts);
  return cudaGetLastError();
}

cudaError_t launch_generate_joint(const JointGenArgs &a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const unsigned g = (unsigned)((a.npix + 127) / 128);
  if (a.fp.n_bands == 4) generate_joint_kernel<4><<<g, 128, 0, s>>>(a);
  else generate_joint_kernel<8><<<g, 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_forward(const ForwardArgs &a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  forward_kernel<<<(unsigned)((a.n + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_empirical_seeds(const EmpSeedArgs &a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const unsigned g = (unsigned)((a.npix + 127) / 128);
  if (a.fp.n_bands == 4) empirical_seeds_kernel<4><<<g, 128, 0, s>>>(a);
  else empirical_seeds_kernel<8><<<g, 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cost(const CostArgs &a, cudaStream_t s) {
  if (a.n <= 0) return cudaSuccess;
  const int block = 128;
  const int64_t grid = (a.n + block - 1) / block;
  if (a.precision == PHOTIC_PREC_DF64) {
    if (a.fp.n_bands == 4) cost_kernel_df<4><<<(unsigned)grid, block, 0, s>>>(a);
    else cost_kernel_df<8><<<(unsigned)grid, block, 0, s>>>(a);
  } else {
    if (a.fp.n_bands == 4) cost_kernel<4><<<(unsigned)grid, block, 0, s>>>(a);
    else cost_kernel<8><<<(unsigned)grid, block, 0, s>>>(a);
  }
  return cudaGetLastError();
}

}  // namespace photic

// ---------------------------------------------------------------------------
// Pipe-throughput probes for the roofline denominators of compute-bound
// kernels: independent FMA chains (FP64 DFMA, FP32 FFMA) and MUFU ex2.
// ---------------------------------------------------------------------------
namespace photic {
namespace {

template <class T>
__global__ void fma_probe(T *out, int iters, T x, T y) {
  T a0 = (T)threadIdx.x * (T)1e-3, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
  T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
  for (int i = 0; i < iters; i++) {
    a0 = fma(a0, x, y); a1 = fma(a1, x, y); a2 = fma(a2, x, y); a3 = fma(a3, x, y);
    a4 = fma(a4, x, y); a5 = fma(a5, x, y); a6 = fma(a6, x, y); a7 = fma(a7, x, y);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

__global__ void mufu_probe(float *out, int iters, float s) {
  float a0 = threadIdx.x * 1e-6f, a1 = a0 + 0.1f, a2 = a0 + 0.2f, a3 = a0 + 0.3f;
  for (int i = 0; i < iters; i++) {
    a0 = exp2f(a0 * s); a1 = exp2f(a1 * s); a2 = exp2f(a2 * s); a3 = exp2f(a3 * s);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3;
}

}  // namespace

cudaError_t measure_peaks(double *fp64_tflops, double *fp32_tflops, double *mufu_tops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int block = 256, grid = sms * 8, n = grid * block;
  void *buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, (size_t)n * sizeof(double));
  if (e != cudaSuccess) return e;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  float ms = 0.f;
  // FP64: 8 DFMA per iteration per thread
  const int it64 = 4096;
  fma_probe<double><<<grid, block>>>((double *)buf, 16, 0.999999, 1e-7);
  cudaEventRecord(t0);
  fma_probe<double><<<grid, block>>>((double *)buf, it64, 0.999999, 1e-7);
  cudaEventRecord(t1);
  cudaEventSynchronize(t1);
  cudaEventElapsedTime(&ms, t0, t1);
  *fp64_tflops = 2.0 * 8.0 * it64 * (double)n / (ms * 1e-3) / 1e12;
  const int it32 = 65536;
  fma_probe<float><<<grid, block>>>((float *)buf, 16, 0.999999f, 1e-7f);
  cudaEventRecord(t0);
  fma_probe<float><<<grid, block>>>((float *)buf, it32, 0.999999f, 1e-7f);
  cudaEventRecord(t1);
  cudaEventSynchronize(t1);
  cudaEventElapsedTime(&ms, t0, t1);
  *fp32_tflops = 2.0 * 8.0 * it32 * (double)n / (ms * 1e-3) / 1e12;
  const int itm = 16384;
  mufu_probe<<<grid, block>>>((float *)buf, 16, 1e-3f);
  cudaEventRecord(t0);
  mufu_probe<<<grid, block>>>((float *)buf, itm, 1e-3f);
  cudaEventRecord(t1);
  cudaEventSynchronize(t1);
  cudaEventElapsedTime(&ms, t0, t1);
  *mufu_tops = 4.0 * itm * (double)n / (ms * 1e-3) / 1e12;
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  e = cudaGetLastError();
  cudaFree(buf);
  return e;
}

cudaError_t launch_depth_sigma_select(const DepthSigmaArgs &a, cudaStream_t s) {
  const unsigned g = (unsigned)((a.npix + 255) / 256);
  if (a.npix > 0) ds_max_kernel<<<g, 256, 0, s>>>(a.depth, a.npix, a.max_bits);
  const int64_t n = (int64_t)kDsMaxIntervals * a.n_samples;
  ds_select_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_depth_sigma_finish(const DepthSigmaArgs &a, cudaStream_t s) {
  ds_table_kernel<<<1, kDsMaxIntervals, 0, s>>>(a);
  if (a.npix > 0) ds_map_kernel<<<(unsigned)((a.npix + 255) / 256), 256, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace photic
