// photic_prec64.cuh -- the FP64 arithmetic policy of the single-scene
// kernels: IEEE double in the reference's operation order for the
// resumable Nelder-Mead of photic_nm.cuh and the cost of photic_fp64.cuh
// (samodel_error / samodel_Rrs, model/samodel.c:2432-2949).  Shared by the
// batched inversion (photic_invert.cu) and the lookup-table pixel loop
// (photic_lut.cu).
#pragma once

#include "photic_fp64.cuh"
#include "photic_kernels.h"
#include "photic_nm.cuh"

namespace photic {

constexpr int kPrecN = 6;  // H, 100B, q, 100P, 100G, 100X

struct PrecF64 {
  using T = double;
  template <int NB>
  using Pixel = PixelF64<NB>;
  struct Details {
    double rrs_error, model_error, bottom_albedo, K_min, iod;
  };
  static __device__ __forceinline__ T zero() { return 0.0; }
  static __device__ __forceinline__ T one() { return 1.0; }
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  static __device__ __forceinline__ T mul2(T a) { return 2.0 * a; }
  static __device__ __forceinline__ T half(T a) { return a * 0.5; }
  // a * c for c in {1/2, 1, 2}: exact
  static __device__ __forceinline__ T scale2(T a, float c) { return a * (double)c; }
  // z / n for the simplex size n, a compile-time constant here
  static __device__ __forceinline__ T div_n(T a, int n) { return fm::div_by(a, (double)n, 1.0 / (double)n); }
  static __device__ __forceinline__ bool lt(T a, T b) { return a < b; }
  static __device__ __forceinline__ bool le(T a, T b) { return a <= b; }
  static __device__ __forceinline__ T eps_step(T s) { return s * 1.0e-6; }
  static __device__ __forceinline__ T eps_scale() { return 1.0e-6; }
  static __device__ __forceinline__ long long trunc10(T y) { return photic::trunc10(y); }
  static __device__ __forceinline__ T from_double(double d) { return d; }
  static __device__ __forceinline__ double to_double(T a) { return a; }
  static __device__ __forceinline__ T var_limit(const InvertArgs &a) { return a.fp.reqmin * (double)kPrecN; }
  static __device__ __forceinline__ T hstart(const InvertArgs &a, int k) {
    double h = a.fp.hstarts[0];
    for (int i = 1; i < kMaxHStarts; i++)
      if (i == k) h = a.fp.hstarts[i];
    return h;
  }
  static __device__ __forceinline__ T h_step(T h) { return 1.25 * h; }
  template <int NB>
  static __device__ __forceinline__ void setup(const InvertArgs &a, const float *r, Pixel<NB> &px) {
    double rd[NB];
#pragma unroll
    for (int b = 0; b < NB; b++) rd[b] = (double)r[b];
    pixel_setup_f64<NB>(a.fp, a.sc, rd, px);
  }
  template <int NB>
  static __device__ __forceinline__ void cold_start(const InvertArgs &a, const Pixel<NB> &px,
                                                    T *start, T *step) {
    cold_start_f64<NB>(a.fp, px, start, step);
  }
  template <int NB>
  static __device__ __forceinline__ T cost(const InvertArgs &a, const Pixel<NB> &px, const T *x) {
    return cost_f64<false, NB>(a.fp, a.sc, px, x, nullptr);
  }
  // One evaluation serves the Nelder-Mead and, at the kept optimum, the
  // products: the kernel evaluates the final point with the other lanes'
  // trial points instead of in a second, divergent cost evaluation.
  static constexpr bool kFused = true;
  template <int NB>
  using Keep = BandKeep<NB>;
  template <int NB>
  static __device__ __forceinline__ T cost_keep(const InvertArgs &a, const Pixel<NB> &px,
                                                const T *x, Keep<NB> &k) {
    return cost_f64<false, NB, Keep<NB>>(a.fp, a.sc, px, x, nullptr, &k);
  }
  // The products of cost_f64<true> (photic_fp64.cuh) from a kept evaluation,
  // the index of optical depth summed in band order.
  template <int NB>
  static __device__ __forceinline__ void details_from_keep(const InvertArgs &a,
                                                           const Keep<NB> &k, T model,
                                                           Details &d) {
    double iod = 0.0;
#pragma unroll
    for (int b = 0; b < NB; b++)
      if (b < a.fp.n_bands) iod = iod + k.rrs_B[b] / k.rrs[b];
    d.rrs_error = k.E;
    d.model_error = model;
    d.bottom_albedo = k.qB;
    d.K_min = k.K_min == 1.0e4 ? 0.0 : k.K_min;
    d.iod = 100.0 * iod / (double)a.fp.n_bands;
  }
  template <int NB>
  static __device__ __forceinline__ void details(const InvertArgs &a, const Pixel<NB> &px,
                                                 const T *x, Details &d) {
    CostDetailsF64 det;
    cost_f64<true, NB>(a.fp, a.sc, px, x, &det);
    d.rrs_error = det.rrs_error;
    d.model_error = det.model_error;
    d.bottom_albedo = det.bottom_albedo;
    d.K_min = det.K_min;
    d.iod = det.iod;
  }
};

// Reference mask test (model/samodel.c:937-941): float tolerance compare
// with the nodata value, or negative reflectance.
__device__ __forceinline__ bool band_masked(float r, float nodata) {
  float diff = __fsub_rn(r, nodata);
  double big = fabs((double)r) < fabs((double)nodata) ? fabs((double)nodata) : fabs((double)r);
  return fabs((double)diff) <= big * (double)1.0e-6f || r < 0.0f;
}

__device__ __forceinline__ void write_masked(const photic_outputs &o, int64_t p) {
  if (o.depth) o.depth[p] = 0.0f;
  if (o.depth_f64) o.depth_f64[p] = 0.0;
  if (o.P) o.P[p] = 0.0f;
  if (o.G) o.G[p] = 0.0f;
  if (o.X) o.X[p] = 0.0f;
  if (o.bottom_albedo) o.bottom_albedo[p] = 0.0f;
  if (o.model_error) o.model_error[p] = 0.0f;
  if (o.rrs_error) o.rrs_error[p] = 0.0f;
  if (o.K_min) o.K_min[p] = 0.0f;
  if (o.iod) o.iod[p] = 0.0f;
  if (o.evals) o.evals[p] = 0;
  if (o.evals_kept) o.evals_kept[p] = 0;
  if (o.status) o.status[p] = PHOTIC_PX_MASKED;
  if (o.params)
    for (int i = 0; i < 6; i++) o.params[p * 6 + i] = 0.0;
}

}  // namespace photic
