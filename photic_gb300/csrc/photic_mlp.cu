// photic_mlp.cu -- the learned warm start: an MLP surrogate
// 6 -> 128 -> 128 -> 128 -> 5 (SiLU) mapping observed Rrs and sun/view zenith
// to (ln P, ln G, ln X, B, H), trained and run with BF16 weights and
// activations and FP32 accumulation on the tcgen05 tensor cores
// (photic_gemm.cu).  Its output only seeds the Nelder-Mead fit, which
// still runs to the plain tolerance; pixels whose seed does not reproduce
// the measured spectrum fall back to the cold start.  No counterpart in
// the reference.
//
// Layer l:  Z_l = A_{l-1} W_l^T + b_l,  A_l = SiLU(Z_l)  (A_0 = normalised
// input padded to 16 features, last layer linear, 5 outputs padded to 16).
// Backward (MSE on standardised targets):
//   dW_l = dZ_l^T A_{l-1},  db_l = colsum(dZ_l),
//   dZ_{l-1} = (dZ_l W_l) * SiLU'(Z_{l-1}).
// Every product is one TN GEMM; the transposed operands it needs are
// formed by small transpose kernels.  Adam keeps FP32 master weights and
// refreshes the BF16 copies (and their transposes) after each step.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "photic_fp64.cuh"
#include "photic_kernels.h"

namespace photic {

namespace {

using bf16 = __nv_bfloat16;

__global__ void featurize_kernel(const float *x, int R, int Rpad, const float *in_mean,
                                 const float *in_std, bf16 *X0) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= Rpad) return;
#pragma unroll
  for (int f = 0; f < kMlpIn; f++) {
    float v = 0.0f;
    if (f < 6 && r < R) v = (x[(size_t)r * 6 + f] - in_mean[f]) / in_std[f];
    X0[(size_t)r * kMlpIn + f] = __float2bfloat16(v);
  }
}

// dst[c][r] = src[r][c] (BF16), rows padded with zeros up to Rpad.
__global__ void transpose_kernel(const bf16 *src, int R, int C, int Rpad, bf16 *dst) {
  __shared__ bf16 tile[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int r = r0 + i, c = c0 + threadIdx.x;
    tile[i][threadIdx.x] = (r < R && c < C) ? src[(size_t)r * C + c] : __float2bfloat16(0.0f);
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int c = c0 + i, r = r0 + threadIdx.x;
    if (c < C && r < Rpad) dst[(size_t)c * Rpad + r] = tile[threadIdx.x][i];
  }
}

// MSE on standardised targets; dY = 2 (Y - t) / (R * 5) as BF16, padding 0.
__global__ void loss_grad_kernel(const float *Y, const float *t, int R, int Rpad,
                                 const float *out_mean, const float *out_std, bf16 *dY,
                                 float *loss) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0.0f;
  if (r < Rpad) {
#pragma unroll
    for (int o = 0; o < kMlpOut; o++) {
      float g = 0.0f;
      if (o < 5 && r < R) {
        const float tn = (t[(size_t)r * 5 + o] - out_mean[o]) / out_std[o];
        const float d = Y[(size_t)r * kMlpOut + o] - tn;
        l += d * d;
        g = 2.0f * d / (float)(R * 5);
      }
      dY[(size_t)r * kMlpOut + o] = __float2bfloat16(g);
    }
  }
  // warp reduction of the loss, one atomic per warp
  for (int off = 16; off; off >>= 1) l += __shfl_down_sync(0xffffffffu, l, off);
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, l / (float)(R * 5));
}

// colsum over rows of a [R][C] BF16 matrix into FP32 g[C].
__global__ void colsum_kernel(const bf16 *m, int R, int C, float *g) {
  const int c = blockIdx.x;
  float s = 0.0f;
  for (int r = threadIdx.x; r < R; r += blockDim.x) s += __bfloat162float(m[(size_t)r * C + c]);
  __shared__ float red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) g[c] = red[0];
}

// out[i][o] = in[o][i] for a small FP32 matrix (weight-gradient layouts).
__global__ void transpose_f32_kernel(const float *in, int rows, int cols, float *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * cols) return;
  const int r = i / cols, c = i % cols;
  out[(size_t)c * rows + r] = in[i];
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters.
__global__ void adam_kernel(float *p, const float *g, float *m, float *v, int n, float lr,
                            float b1, float b2, float eps, float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.0f - b1) * gi;
  const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// BF16 copies of the weights: W1b [128][16], W2b, W3b [128][128], W4b [16][128]
// and the transposes used by the input-gradient products.
__global__ void refresh_kernel(const float *P, bf16 *W1b, bf16 *W2b, bf16 *W3b, bf16 *W4b,
                               bf16 *W2t, bf16 *W3t, bf16 *W4t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float *W1 = P + kOffW1, *W2 = P + kOffW2, *W3 = P + kOffW3, *W4 = P + kOffW4;
  if (i < kMlpH * kMlpIn) W1b[i] = __float2bfloat16(W1[i]);
  if (i < kMlpH * kMlpH) {
    const int r = i / kMlpH, c = i % kMlpH;
    W2b[i] = __float2bfloat16(W2[i]);
    W3b[i] = __float2bfloat16(W3[i]);
    W2t[(size_t)c * kMlpH + r] = __float2bfloat16(W2[i]);
    W3t[(size_t)c * kMlpH + r] = __float2bfloat16(W3[i]);
  }
  if (i < kMlpOut * kMlpH) {
    const int r = i / kMlpH, c = i % kMlpH;
    W4b[i] = __float2bfloat16(W4[i]);
    W4t[(size_t)c * kMlpOut + r] = __float2bfloat16(W4[i]);
  }
}

__global__ void denorm_kernel(const float *Y, int R, const float *out_mean, const float *out_std,
                              float *y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
#pragma unroll
  for (int o = 0; o < 5; o++) y[(size_t)r * 5 + o] = Y[(size_t)r * kMlpOut + o] * out_std[o] + out_mean[o];
}

// Forward model of one band in single precision for the seed polish
// (the seed only has to land near a minimum; nelmin then runs in FP64):
// z = (ln P, ln G, ln X, B, H), one bottom type with q = 1.  The band
// constants come as floats (SceneF32), so the loop has no double
// conversions.
__device__ __forceinline__ float forward_band_f32(const SceneF32 &sf, int b, const float (&z)[5],
                                                  float pw) {
  const float P = __expf(z[0]), G = __expf(z[1]), X = __expf(z[2]);
  const float B = fabsf(z[3]), H = fabsf(z[4]);
  const float rho = B * sf.refl[b];
  const float a = sf.aw[b] + (sf.a0[b] + sf.a1[b] * z[0]) * P + G * sf.eS[b];
  const float bb = sf.bbw[b] + X * pw;
  const float u = bb / (a + bb);
  const float K = fminf(fmaxf(a + bb, 0.0f), 2.5f);
  const float rdp = (0.084f + 0.170f * u) * u;
  const float duc = 1.03f * sqrtf(1.0f + 2.4f * u);
  const float dub = 1.04f * sqrtf(1.0f + 5.4f * u);
  const float rc = rdp * (1.0f - __expf(-(sf.sec_sun + duc * sf.sec_view) * K * H));
  const float rb = rho * 0.3183098862f * __expf(-(sf.sec_sun + dub * sf.sec_view) * K * H);
  const float r = rc + rb;
  return 0.5f * r / (1.0f - 1.5f * r);
}

// Sum of squares of the polish residuals: the spectral misfit in units of
// the noise sigma, plus a weak pull towards the network's prediction z0
// that picks one point of the (underdetermined) solution set.  The pull is
// kept small (weight 0.003): the closer the seed lies to the measured
// spectrum, the sooner the plain-tolerance fit from it converges (most
// seeded fits then end after their first convergence test).
template <int NB>
__device__ __forceinline__ float polish_cost(const SceneF32 &sf, int nb, const float (&z)[5],
                                             const float (&z0)[5], const float (&pw)[NB],
                                             const float (&rs)[NB], float inv_sigma,
                                             float w, float (&e)[NB + 5]) {
  float s = 0.0f;
#pragma unroll
  for (int b = 0; b < NB; b++) {
    e[b] = 0.0f;
    if (b < nb) e[b] = (forward_band_f32(sf, b, z, pw[b]) - rs[b]) * inv_sigma;
    s += e[b] * e[b];
  }
#pragma unroll
  for (int i = 0; i < 5; i++) {
    e[NB + i] = w * (z[i] - z0[i]);
    s += e[NB + i] * e[NB + i];
  }
  return s;
}

// Levenberg-Marquardt on the 5 seed parameters, all in FP32: forward-
// difference Jacobian, normal equations scaled to a unit diagonal (which
// takes the parameters' disparate units out of the conditioning), damping
// lambda on the scaled system (Marquardt's lambda * diag), Cholesky solve;
// lambda divided by 4 on an accepted step and multiplied by 4 on a
// rejected one.  Returns the final spectral misfit (sum of squares over
// the bands, in units of sigma^2).
template <int NB>
__device__ __forceinline__ float polish_seed(const SceneF32 &sf, int nb, const float (&pw)[NB],
                             const float (&rs)[NB], float inv_sigma, int iters, float (&z)[5]) {
  constexpr int M = NB + 5;
  const float w = 0.003f;
  float z0[5], e[M], et[M], J[M][5];
#pragma unroll
  for (int i = 0; i < 5; i++) z0[i] = z[i];
  float S = polish_cost<NB>(sf, nb, z, z0, pw, rs, inv_sigma, w, e);
  float lambda = 1.0e-3f;
  bool need_j = true;
  for (int it = 0; it < iters; it++) {
    if (need_j) {
#pragma unroll
      for (int i = 0; i < 5; i++) {
        const float h = 1.0e-3f * fmaxf(1.0f, fabsf(z[i]));
        float zi[5];
#pragma unroll
        for (int k = 0; k < 5; k++) zi[k] = z[k];
        zi[i] += h;
        polish_cost<NB>(sf, nb, zi, z0, pw, rs, inv_sigma, w, et);
        const float inv_h = 1.0f / h;
#pragma unroll
        for (int m = 0; m < M; m++) J[m][i] = (et[m] - e[m]) * inv_h;
      }
      need_j = false;
    }
    float A[5][5], g[5], sc[5];
#pragma unroll
    for (int i = 0; i < 5; i++) {
      float gs = 0.0f;
#pragma unroll
      for (int m = 0; m < M; m++) gs += J[m][i] * e[m];
      g[i] = gs;
#pragma unroll
      for (int k = 0; k <= i; k++) {
        float s = 0.0f;
#pragma unroll
        for (int m = 0; m < M; m++) s += J[m][i] * J[m][k];
        A[i][k] = s;
      }
    }
#pragma unroll
    for (int i = 0; i < 5; i++) sc[i] = rsqrtf(A[i][i] + 1.0e-30f);
#pragma unroll
    for (int i = 0; i < 5; i++) {
      g[i] *= sc[i];
#pragma unroll
      for (int k = 0; k <= i; k++) A[i][k] *= sc[i] * sc[k];
      A[i][i] += lambda;
    }
    // Cholesky of the scaled, damped matrix (lower triangle in place)
    bool ok = true;
#pragma unroll
    for (int i = 0; i < 5; i++) {
#pragma unroll
      for (int k = 0; k <= i; k++) {
        float s = A[i][k];
#pragma unroll
        for (int m = 0; m < k; m++) s -= A[i][m] * A[k][m];
        if (i == k) {
          if (!(s > 0.0f)) ok = false;
          A[i][i] = sqrtf(fmaxf(s, 1.0e-30f));
        } else {
          A[i][k] = s / A[k][k];
        }
      }
    }
    if (!ok) {
      lambda *= 4.0f;
      continue;
    }
    float y[5], d[5];
#pragma unroll
    for (int i = 0; i < 5; i++) {
      float s = -g[i];
#pragma unroll
      for (int m = 0; m < i; m++) s -= A[i][m] * y[m];
      y[i] = s / A[i][i];
    }
#pragma unroll
    for (int i = 4; i >= 0; i--) {
      float s = y[i];
#pragma unroll
      for (int m = i + 1; m < 5; m++) s -= A[m][i] * d[m];
      d[i] = s / A[i][i];
    }
    float zt[5];
#pragma unroll
    for (int i = 0; i < 5; i++) zt[i] = z[i] + d[i] * sc[i];
    const float St = polish_cost<NB>(sf, nb, zt, z0, pw, rs, inv_sigma, w, et);
    if (St < S) {
      S = St;
#pragma unroll
      for (int i = 0; i < 5; i++) z[i] = zt[i];
#pragma unroll
      for (int m = 0; m < M; m++) e[m] = et[m];
      lambda *= 0.25f;
      need_j = true;
    } else {
      lambda *= 4.0f;
    }
  }
  float fit = 0.0f;
#pragma unroll
  for (int b = 0; b < NB; b++) fit += e[b] * e[b];
  return fit;
}

// Seeds for nelmin from the surrogate's prediction (optionally polished
// by a few Levenberg-Marquardt steps on the spectral misfit), and the
// fallback test: the seed's modelled spectrum must match the measured one
// to within resid_max (RMS over bands), otherwise the pixel keeps the cold
// start.
template <int NB>
__global__ void seeds_kernel(const __grid_constant__ SeedArgs a) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  const int nb = a.fp.n_bands;
  double *sd = a.seeds + p * 6;
  double r[NB];
  bool bad = false;
#pragma unroll
  for (int b = 0; b < NB; b++) {
    r[b] = b < nb ? (double)a.rrs[p * nb + b] : 0.0;
    if (b < nb && !(r[b] >= 0.0)) bad = true;
  }
  PixelF64<NB> px;
  if (!bad) pixel_setup_f64<NB>(a.fp, a.sc, r, px);
  float z[5];
  if (a.y != nullptr) {
    const float *yp = a.y + p * 5;
    z[0] = yp[0];
    z[1] = yp[1];
    z[2] = yp[2];
    z[3] = fmaxf(yp[3], 0.001f);
    z[4] = fmaxf(yp[4], 0.1f);
  } else {
    // no network: the reference's cold start of B, P, G, X from the
    // measured spectrum, depth h_guess
    double st[6], sp[6];
    st[1] = st[3] = st[4] = st[5] = 0.0;
    if (!bad) cold_start_f64<NB>(a.fp, px, st, sp);
    z[0] = (float)log(0.01 * st[3]);
    z[1] = (float)log(0.01 * st[4]);
    z[2] = (float)log(0.01 * st[5]);
    z[3] = fmaxf((float)(0.01 * st[1]), 0.001f);
    z[4] = fmaxf((float)a.h_guess, 0.1f);
  }
  if (!bad && a.polish_iters > 0 && isfinite(z[0] + z[1] + z[2] + z[3] + z[4])) {
    // up to three attempts: the prediction, then its depth scaled by 0.4
    // and by 2.5 (the depth is the least determined parameter); the first
    // that fits the spectrum to 0.8 resid_max wins, else the best fit
    float pw[NB], rs[NB];
#pragma unroll
    for (int b = 0; b < NB; b++) {
      pw[b] = (float)px.pw[b];
      rs[b] = (float)r[b];
    }
    const float inv_sigma = (float)(3.0 / a.resid_max);
    const float accept = 0.64f * 9.0f * (float)nb;  // (0.8 resid_max / sigma)^2 * bands
    const float hs[3] = {1.0f, 0.4f, 2.5f};
    float best[5] = {z[0], z[1], z[2], z[3], z[4]}, best_fit = 3.0e38f;
    for (int k = 0; k < 3; k++) {
      float zk[5] = {z[0], z[1], z[2], z[3], fmaxf(z[4] * hs[k], 0.1f)};
      const float f = polish_seed<NB>(a.sf, nb, pw, rs, inv_sigma, a.polish_iters, zk);
      if (f < best_fit) {
        best_fit = f;
#pragma unroll
        for (int i = 0; i < 5; i++) best[i] = zk[i];
      }
      if (best_fit <= accept) break;
    }
#pragma unroll
    for (int i = 0; i < 5; i++) z[i] = best[i];
  }
  const double P = exp((double)z[0]), G = exp((double)z[1]), X = exp((double)z[2]);
  double B = fabs((double)z[3]), H = fabs((double)z[4]);
  if (B < 0.001) B = 0.001;
  if (H < 0.1) H = 0.1;
  double x[6] = {H, 100.0 * B, 1.0, 100.0 * P, 100.0 * G, 100.0 * X};
  double resid = 1.0e30;
  if (!bad) {
    CostDetailsF64 det;
    cost_f64<true, NB>(a.fp, a.sc, px, x, &det);
    double s2 = 0.0;
    for (int b = 0; b < nb; b++) {
      const double d = det.Rm[b] - r[b];
      s2 += d * d;
    }
    resid = sqrt(s2 / (double)nb);
  }
  const bool warm = resid <= a.resid_max;
  if (a.resid) a.resid[p] = (float)resid;
#pragma unroll
  for (int i = 0; i < 6; i++) sd[i] = x[i];
  if (!warm) sd[0] = __longlong_as_double(0x7ff8000000000000LL);  // NaN: cold start
}

__global__ void features_from_rrs_kernel(const float *rrs, int64_t npix, int nb, float th_sun,
                                         float th_view, float *x) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  for (int b = 0; b < 4; b++) x[p * 6 + b] = b < nb ? rrs[p * nb + b] : 0.0f;
  x[p * 6 + 4] = th_sun;
  x[p * 6 + 5] = th_view;
}

}  // namespace

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------

static int gemm(const void *A, int lda, const void *B, int ldb, int M, int N, int K, int epi,
                float *C, int ldc, void *O, int ldo, float *Z, int ldz, const float *bias,
                unsigned int *err, cudaStream_t s, float *splitk = nullptr) {
  GemmArgs g{};
  g.ksplit = splitk ? kMlpSplitK : 1;
  g.partial = splitk;
  g.A = A;
  g.B = B;
  g.lda = lda;
  g.ldb = ldb;
  g.M = M;
  g.N = N;
  g.K = K;
  g.C = C;
  g.ldc = ldc;
  g.O = O;
  g.ldo = ldo;
  g.Z = Z;
  g.ldz = ldz;
  g.bias = bias;
  g.error = err;
  g.lbo = 128;
  g.sbo = 1024;
  g.epi = epi;
  return launch_gemm(g, s) == cudaSuccess ? 0 : 1;
}

cudaError_t mlp_refresh(const MlpState &st, cudaStream_t s) {
  refresh_kernel<<<(kMlpH * kMlpH + 255) / 256, 256, 0, s>>>(st.P, st.W1b, st.W2b, st.W3b,
                                                             st.W4b, st.W2t, st.W3t, st.W4t);
  return cudaGetLastError();
}

// Forward pass over Rpad rows (multiple of 128) of features x [R][6].
cudaError_t mlp_forward(const MlpState &st, const float *x, int R, int Rpad, MlpWork &w,
                        unsigned int *err, cudaStream_t s) {
  featurize_kernel<<<(Rpad + 255) / 256, 256, 0, s>>>(x, R, Rpad, st.in_mean, st.in_std, w.X0);
  int bad = 0;
  bad |= gemm(w.X0, kMlpIn, st.W1b, kMlpIn, Rpad, kMlpH, kMlpIn, EPI_BIAS_SILU, nullptr, 0, w.A1,
              kMlpH, w.Z1, kMlpH, st.P + kOffB1, err, s);
  bad |= gemm(w.A1, kMlpH, st.W2b, kMlpH, Rpad, kMlpH, kMlpH, EPI_BIAS_SILU, nullptr, 0, w.A2,
              kMlpH, w.Z2, kMlpH, st.P + kOffB2, err, s);
  bad |= gemm(w.A2, kMlpH, st.W3b, kMlpH, Rpad, kMlpH, kMlpH, EPI_BIAS_SILU, nullptr, 0, w.A3,
              kMlpH, w.Z3, kMlpH, st.P + kOffB3, err, s);
  bad |= gemm(w.A3, kMlpH, st.W4b, kMlpH, Rpad, kMlpOut, kMlpH, EPI_BIAS_F32, w.Y, kMlpOut,
              nullptr, 0, nullptr, 0, st.P + kOffB4, err, s);
  if (bad) return cudaErrorLaunchFailure;
  return cudaGetLastError();
}

static void tr(const bf16 *src, int R, int C, int Rpad, bf16 *dst, cudaStream_t s) {
  dim3 grid((unsigned)((Rpad + 31) / 32), (unsigned)((C + 31) / 32));
  transpose_kernel<<<grid, dim3(32, 8), 0, s>>>(src, R, C, Rpad, dst);
}

// Forward + backward; gradients (same layout as the parameters) into w.grad.
cudaError_t mlp_backward(const MlpState &st, const float *x, const float *t, int R, int Rpad,
                         MlpWork &w, float *loss, unsigned int *err, cudaStream_t s) {
  cudaError_t e = mlp_forward(st, x, R, Rpad, w, err, s);
  if (e != cudaSuccess) return e;
  float *g = w.grad;
  loss_grad_kernel<<<(Rpad + 255) / 256, 256, 0, s>>>(w.Y, t, R, Rpad, st.out_mean, st.out_std,
                                                      w.dY, loss);
  int bad = 0;
  // layer 4: dW4 = dY^T A3 (computed as (A3^T dY)^T), db4 = colsum(dY)
  tr(w.A3, Rpad, kMlpH, Rpad, w.T1, s);
  tr(w.dY, Rpad, kMlpOut, Rpad, w.T2, s);
  bad |= gemm(w.T1, Rpad, w.T2, Rpad, kMlpH, kMlpOut, Rpad, EPI_F32, w.G4t, kMlpOut, nullptr, 0,
              nullptr, 0, nullptr, err, s, w.splitk);
  transpose_f32_kernel<<<(kMlpH * kMlpOut + 255) / 256, 256, 0, s>>>(w.G4t, kMlpH, kMlpOut,
                                                                     g + kOffW4);
  colsum_kernel<<<kMlpOut, 256, 0, s>>>(w.dY, Rpad, kMlpOut, g + kOffB4);
  // dZ3 = (dY W4) * SiLU'(Z3)
  bad |= gemm(w.dY, kMlpOut, st.W4t, kMlpOut, Rpad, kMlpH, kMlpOut, EPI_DSILU, nullptr, 0,
              w.dZ, kMlpH, w.Z3, kMlpH, nullptr, err, s);
  // layer 3
  tr(w.dZ, Rpad, kMlpH, Rpad, w.T2, s);
  tr(w.A2, Rpad, kMlpH, Rpad, w.T1, s);
  bad |= gemm(w.T2, Rpad, w.T1, Rpad, kMlpH, kMlpH, Rpad, EPI_F32, g + kOffW3, kMlpH, nullptr, 0,
              nullptr, 0, nullptr, err, s, w.splitk);
  colsum_kernel<<<kMlpH, 256, 0, s>>>(w.dZ, Rpad, kMlpH, g + kOffB3);
  bad |= gemm(w.dZ, kMlpH, st.W3t, kMlpH, Rpad, kMlpH, kMlpH, EPI_DSILU, nullptr, 0, w.dZ2,
              kMlpH, w.Z2, kMlpH, nullptr, err, s);
  // layer 2
  tr(w.dZ2, Rpad, kMlpH, Rpad, w.T2, s);
  tr(w.A1, Rpad, kMlpH, Rpad, w.T1, s);
  bad |= gemm(w.T2, Rpad, w.T1, Rpad, kMlpH, kMlpH, Rpad, EPI_F32, g + kOffW2, kMlpH, nullptr, 0,
              nullptr, 0, nullptr, err, s, w.splitk);
  colsum_kernel<<<kMlpH, 256, 0, s>>>(w.dZ2, Rpad, kMlpH, g + kOffB2);
  bad |= gemm(w.dZ2, kMlpH, st.W2t, kMlpH, Rpad, kMlpH, kMlpH, EPI_DSILU, nullptr, 0, w.dZ,
              kMlpH, w.Z1, kMlpH, nullptr, err, s);
  // layer 1 (no input gradient needed)
  tr(w.dZ, Rpad, kMlpH, Rpad, w.T2, s);
  tr(w.X0, Rpad, kMlpIn, Rpad, w.T1, s);
  bad |= gemm(w.T2, Rpad, w.T1, Rpad, kMlpH, kMlpIn, Rpad, EPI_F32, g + kOffW1, kMlpIn, nullptr,
              0, nullptr, 0, nullptr, err, s, w.splitk);
  colsum_kernel<<<kMlpH, 256, 0, s>>>(w.dZ, Rpad, kMlpH, g + kOffB1);
  if (bad) return cudaErrorLaunchFailure;
  return cudaGetLastError();
}

cudaError_t mlp_adam(const MlpState &st, const MlpWork &w, float lr, int step, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1.0e-8f;
  const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
  adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, s>>>(st.P, w.grad, st.M, st.V, kMlpParams, lr,
                                                       b1, b2, eps, bc1, bc2);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return mlp_refresh(st, s);
}

cudaError_t mlp_denorm(const MlpState &st, const MlpWork &w, int R, float *y, cudaStream_t s) {
  denorm_kernel<<<(R + 255) / 256, 256, 0, s>>>(w.Y, R, st.out_mean, st.out_std, y);
  return cudaGetLastError();
}

cudaError_t mlp_features(const float *rrs, int64_t npix, int nb, float th_sun, float th_view,
                         float *x, cudaStream_t s) {
  if (npix <= 0) return cudaSuccess;
  features_from_rrs_kernel<<<(unsigned)((npix + 255) / 256), 256, 0, s>>>(rrs, npix, nb, th_sun,
                                                                          th_view, x);
  return cudaGetLastError();
}

cudaError_t mlp_seeds(const SeedArgs &a, cudaStream_t s) {
  if (a.npix <= 0) return cudaSuccess;
  const unsigned g = (unsigned)((a.npix + 127) / 128);
  if (a.fp.n_bands == 4) seeds_kernel<4><<<g, 128, 0, s>>>(a);
  else seeds_kernel<8><<<g, 128, 0, s>>>(a);
  return cudaGetLastError();
}

}  // namespace photic
