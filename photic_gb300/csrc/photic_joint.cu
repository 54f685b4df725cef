// photic_joint.cu -- the temporal joint fit: k scenes of one pixel share
// depth (and, in the reference layout, bottom albedo), each scene keeps its
// own water column (P, G, X) and sun angle (model/samodel.c:2463-2491; the
// start vector of model/samodel.c:2249-2353 with n_scenes = k).
//
// Pixels arrive as CSR over observations (one observation = one scene of one
// pixel).  Ragged scene counts k = 1..8 give simplices of n = 3 + 3k
// (reference layout) or 1 + 4k (per-scene bottom albedo) unknowns, so the
// pixels are first binned by k on the device (count, scan, scatter) and one
// persistent kernel per k then works through its bin -- lanes of a warp
// never run different simplex sizes.  No host round trip is needed between
// the stages, so the whole call can be captured in a CUDA graph.
//
// The arithmetic is IEEE double in the reference's operation order, like
// the FP64 single-scene kernel.  A simplex of up to 34 x 33 values does not
// fit in registers or shared memory per lane; it lives in thread-local
// memory (L1/L2 backed) -- the FP64 pipe, not memory, bounds this kernel.
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_fp64.cuh"
#include "photic_kernels.h"
#include "photic_nm.cuh"

namespace photic {

namespace {

struct PrecJ {
  using T = double;
  static __device__ __forceinline__ T zero() { return 0.0; }
  static __device__ __forceinline__ T one() { return 1.0; }
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  static __device__ __forceinline__ T mul2(T a) { return 2.0 * a; }
  static __device__ __forceinline__ T half(T a) { return a * 0.5; }
  static __device__ __forceinline__ T scale2(T a, float c) { return a * (double)c; }
  static __device__ __forceinline__ T div_n(T a, int n) { return fm::div_by(a, (double)n, 1.0 / (double)n); }
  static __device__ __forceinline__ bool lt(T a, T b) { return a < b; }
  static __device__ __forceinline__ bool le(T a, T b) { return a <= b; }
  static __device__ __forceinline__ T eps_step(T s) { return s * 1.0e-6; }
  static __device__ __forceinline__ T eps_scale() { return 1.0e-6; }
  static __device__ __forceinline__ long long trunc10(T y) { return photic::trunc10(y); }
};

template <int LAYOUT, int K>
struct Dims {
  static constexpr int N = LAYOUT == PHOTIC_LAYOUT_REFERENCE ? 3 + 3 * K : 1 + 4 * K;
};

// Per-pixel constants of the k scenes.
template <int K, int NB>
struct JPixel {
  double rrs[K][NB];
  double pw[K][NB];
  double sec_sun[K];
  double r490[K], r550[K], r640[K];
  double mean;
};

template <int K, int NB>
__device__ __forceinline__ void jsetup(const JointArgs &a, int64_t o0, JPixel<K, NB> &px) {
  const FitParams &fp = a.fp;
  const int nb = fp.n_bands;
  double tot = 0.0;
  for (int s = 0; s < K; s++) {
#pragma unroll
    for (int b = 0; b < NB; b++) {
      px.rrs[s][b] = 0.0;
      if (b < nb) {
        px.rrs[s][b] = (double)a.rrs[(o0 + s) * nb + b];
        tot = tot + px.rrs[s][b];
      }
    }
    double r440 = interp_plan<NB>(fp.plan[0], px.rrs[s]);
    px.r490[s] = interp_plan<NB>(fp.plan[1], px.rrs[s]);
    px.r550[s] = interp_plan<NB>(fp.plan[2], px.rrs[s]);
    px.r640[s] = interp_plan<NB>(fp.plan[3], px.rrs[s]);
    if (r440 < 0.0) r440 = 0.0001;
    const double chi = r440 / px.r490[s];
    double Y = 3.44 * (1.0 - 3.17 * fm::exp_t(-2.01 * chi));
    if (Y < 0.0) Y = 0.0;
    if (Y > 2.5) Y = 2.5;
#pragma unroll
    for (int b = 0; b < NB; b++)
      if (b < nb) px.pw[s][b] = pow(a.sc.ratio440[b], Y);
    // subsurface sun zenith in degrees -> secant (model/samodel.c:543-548)
    double th = a.theta_sun[o0 + s];
    th *= 3.141592653589793 / 180.0;
    px.sec_sun[s] = 1.0 / cos(th);
  }
  px.mean = tot / (double)(K * nb);
}

struct JDetails {
  double rrs_error, model_error, bottom_albedo, K_min, iod;
};

// samodel_error (model/samodel.c:2432-2759) with n_scenes = K, one region,
// one bottom type, in the reference's loop order (scene, then band).
template <int LAYOUT, int K, int NB, bool kDetails>
__device__ __forceinline__ double jcost(const JointArgs &a, const JPixel<K, NB> &px,
                                        const double *x, JDetails *det) {
  const FitParams &fp = a.fp;
  const SceneConsts &sc = a.sc;
  const int nb = fp.n_bands;
  const double H = fabs(x[0]);
  double err = 0.0, iod = 0.0, qB = 0.0, Kall = 1.0e4;
  double kmin[K];
  for (int s = 0; s < K; s++) {
    double P, G, X;
    if (LAYOUT == PHOTIC_LAYOUT_REFERENCE) {
      const double B = 0.01 * fabs(x[1]);
      const double qa = fabs(x[2]);
      qB = fm::self_ratio(qa) * B;
      P = 0.01 * fabs(x[3 + 3 * s]);
      G = 0.01 * fabs(x[4 + 3 * s]);
      X = 0.01 * fabs(x[5 + 3 * s]);
    } else {
      qB = 1.0 * (0.01 * fabs(x[1 + 4 * s]));
      P = 0.01 * fabs(x[2 + 4 * s]);
      G = 0.01 * fabs(x[3 + 4 * s]);
      X = 0.01 * fabs(x[4 + 4 * s]);
    }
    const double lnP = log(P);
    double km = 1.0e4;
#pragma unroll
    for (int b = 0; b < NB; b++) {
      if (b < nb) {
        const double rho = qB * sc.refl[b];
        const double a_phi = (sc.a0[b] + sc.a1[b] * lnP) * P;
        const double a_g = G * sc.eS[b];
        const double aa = sc.aw[b] + a_phi + a_g;
        const double bb = sc.bbw[b] + X * px.pw[s][b];
        const double u = bb / (aa + bb);
        double Kb = aa + bb;
        if (Kb < 0.0) Kb = 0.0;
        if (Kb > 2.5) Kb = 2.5;
        const double rrs_dp = (0.084 + 0.170 * u) * u;
        const double DuC = 1.03 * sqrt(1.0 + 2.4 * u);
        const double DuB = 1.04 * sqrt(1.0 + 5.4 * u);
        double M = px.sec_sun[s] + DuC * sc.sec_view;
        const double rrs_C = rrs_dp * (1.0 - fm::exp_t(-M * Kb * H));
        M = px.sec_sun[s] + DuB * sc.sec_view;
        const double rrs_B = fm::div_by(rho, kPi, fm::kInvPi) * fm::exp_t(-M * Kb * H);
        const double rrs = rrs_C + rrs_B;
        const double Rm = 0.5 * rrs / (1.0 - 1.5 * rrs);
        const double d = Rm - px.rrs[s][b];
        err = err + d * d;
        if (__double2float_rn(Kb) != 0.0f && Kb < km) km = Kb;
        if (kDetails) {
          iod = iod + rrs_B / rrs;
          if (__double2float_rn(Kb) != 0.0f && Kb < Kall) Kall = Kb;
        }
      }
    }
    kmin[s] = km;
  }
  const double E = 100.0 * sqrt(fm::div_count(err, K * nb)) / px.mean;
  double Ke = 0.0;
  for (int s = 0; s < K; s++) Ke = Ke + k_penalty_f64(fp.kp, H, kmin[s]);
  if (kmin[K - 1] > 0.7) {
    const double d = 4.0 * (kmin[K - 1] - 0.7);
    Ke = Ke + 100.0 * (d * d);
  }
  double model = 80.0 * E + 15.0 * Ke;
  model = fm::div_by(model, 120.0, fm::kInv120);
  if (kDetails) {
    det->rrs_error = E;
    det->model_error = model;
    det->bottom_albedo = qB;
    det->K_min = Kall == 1.0e4 ? 0.0 : Kall;
    det->iod = 100.0 * iod / (double)(K * nb);
  }
  return model;
}

// Cold start (model/samodel.c:2249-2353) for k scenes; depth filled later.
template <int LAYOUT, int K, int NB, int N>
__device__ __forceinline__ void jcold(const JointArgs &a, const JPixel<K, NB> &px, double *start,
                                      double *step) {
  const double c5 = 100.0 * 30.0 * a.fp.aw640;
  if (LAYOUT == PHOTIC_LAYOUT_REFERENCE) {
    double m490 = 0.0;
    for (int s = 0; s < K; s++) m490 += px.r490[s];
    m490 /= (double)1 * K;
    start[1] = 100.0 * 4.0 * m490;
    step[1] = 1.5 * start[1];
    start[2] = 1.0;
    step[2] = 0.5 * start[2];
    for (int s = 0; s < K; s++) {
      const int o = 3 + 3 * s;
      start[o] = 100.0 * 0.072 * pow(px.r490[s] / px.r550[s], -1.7);
      start[o + 1] = 1.5 * start[o];
      start[o + 2] = c5 * px.r640[s];
      step[o] = 2.0 * start[o];
      step[o + 1] = 2.0 * start[o + 1];
      step[o + 2] = 2.0 * start[o + 2];
    }
  } else {
    for (int s = 0; s < K; s++) {
      const int o = 1 + 4 * s;
      start[o] = 100.0 * 4.0 * px.r490[s];
      step[o] = 1.5 * start[o];
      start[o + 1] = 100.0 * 0.072 * pow(px.r490[s] / px.r550[s], -1.7);
      start[o + 2] = 1.5 * start[o + 1];
      start[o + 3] = c5 * px.r640[s];
      step[o + 1] = 2.0 * start[o + 1];
      step[o + 2] = 2.0 * start[o + 2];
      step[o + 3] = 2.0 * start[o + 3];
    }
  }
}

template <int LAYOUT, int K, int NB>
__global__ void __launch_bounds__(128) joint_kernel(const __grid_constant__ JointArgs a) {
  constexpr int N = Dims<LAYOUT, K>::N;
  const FitParams &fp = a.fp;
  const photic_outputs &o = a.out;
  const int bin = K - 1;
  const int32_t count = a.bin_count[bin];
  const int32_t first = a.bin_start[bin];

  double vmem[(N + 1) * N], fmem[N + 1], best[N];
  NmLane<N, PrecJ, 1> m;
  m.v = vmem;
  m.f = fmem;
  JPixel<K, NB> px;
  const double var_limit = fp.reqmin * (double)N;
  const double early = fp.early_exit_per_scene * (double)(float)K;
  const int32_t guard_cap = (fp.n_hstarts + 1) * (fp.kcount + 8 * N + 16);

  for (;;) {
    const unsigned long long t = atomicAdd(&a.queues[bin], 1ull);
    if (t >= (unsigned long long)count) break;
    const int64_t p = a.list[first + (int64_t)t];
    const int64_t o0 = a.offsets[p];
    // nodata / negative in any band of any scene (model/samodel.c:933-947)
    bool masked = false;
    for (int s = 0; s < K; s++)
      for (int b = 0; b < fp.n_bands; b++) {
        const float r = a.rrs[(o0 + s) * fp.n_bands + b];
        const float diff = __fsub_rn(r, fp.nodata);
        const double big = fabs((double)r) < fabs((double)fp.nodata) ? fabs((double)fp.nodata)
                                                                     : fabs((double)r);
        if (fabs((double)diff) <= big * (double)1.0e-6f || r < 0.0f) masked = true;
      }
    if (masked) {
      if (o.depth) o.depth[p] = 0.0f;
      if (o.depth_f64) o.depth_f64[p] = 0.0;
      if (o.bottom_albedo) o.bottom_albedo[p] = 0.0f;
      if (o.model_error) o.model_error[p] = 0.0f;
      if (o.rrs_error) o.rrs_error[p] = 0.0f;
      if (o.K_min) o.K_min[p] = 0.0f;
      if (o.iod) o.iod[p] = 0.0f;
      if (o.evals) o.evals[p] = 0;
      if (o.evals_kept) o.evals_kept[p] = 0;
      if (o.status) o.status[p] = PHOTIC_PX_MASKED;
      for (int s = 0; s < K; s++) {
        if (o.P) o.P[o0 + s] = 0.0f;
        if (o.G) o.G[o0 + s] = 0.0f;
        if (o.X) o.X[o0 + s] = 0.0f;
      }
      continue;
    }
    jsetup<K, NB>(a, o0, px);
    int32_t total = 0, kept_evals = 0, kept_start = 0, kept_fault = 0, guard = 0;
    double lowest = 1.0e4;
    for (int i = 0; i < N; i++) best[i] = 0.0;
    bool bad = false;
    for (int k = 0; k < fp.n_hstarts && !bad; k++) {
      jcold<LAYOUT, K, NB, N>(a, px, m.start, m.step);
      double h = fp.hstarts[0];
      for (int i = 1; i < kMaxHStarts; i++)
        if (i == k) h = fp.hstarts[i];
      m.start[0] = h;
      m.step[0] = 1.25 * m.start[0];
      m.begin(var_limit, fp.konvge, fp.kcount);
      bool done = false;
      while (!done) {
        const double y = jcost<LAYOUT, K, NB, false>(a, px, m.x, nullptr);
        if (++guard > guard_cap) {
          atomicOr(a.error, PHOTIC_DEVERR_EVAL_CAP);
          bad = true;
          break;
        }
        done = m.step_machine(y);
      }
      if (bad) break;
      const double ynewlo = m.F(m.lo);
      total += m.icount;
      if (ynewlo < lowest) {
        lowest = ynewlo;
        for (int i = 0; i < N; i++) best[i] = m.xmin[i];
        kept_evals = m.icount;
        kept_start = k;
        kept_fault = m.ifault;
        if (lowest < early) break;  // model/samodel.c:2404
      }
    }
    if (bad) {
      if (o.status) o.status[p] = PHOTIC_PX_INVALID;
      continue;
    }
    JDetails det;
    jcost<LAYOUT, K, NB, true>(a, px, best, &det);
    const double H = fabs(best[0]);
    if (o.depth) o.depth[p] = (float)H;
    if (o.depth_f64) o.depth_f64[p] = H;
    if (o.bottom_albedo) o.bottom_albedo[p] = (float)det.bottom_albedo;
    if (o.model_error) o.model_error[p] = (float)det.model_error;
    if (o.rrs_error) o.rrs_error[p] = (float)det.rrs_error;
    if (o.K_min) o.K_min[p] = (float)det.K_min;
    if (o.iod) o.iod[p] = (float)det.iod;
    if (o.evals) o.evals[p] = total;
    if (o.evals_kept) o.evals_kept[p] = kept_evals;
    if (o.status)
      o.status[p] = PHOTIC_PX_FITTED | (kept_fault == 0 ? PHOTIC_PX_CONVERGED : 0) |
                    (kept_start << 16);
    for (int s = 0; s < K; s++) {
      const int ip = LAYOUT == PHOTIC_LAYOUT_REFERENCE ? 3 + 3 * s : 2 + 4 * s;
      if (o.P) o.P[o0 + s] = (float)(0.01 * fabs(best[ip]));
      if (o.G) o.G[o0 + s] = (float)(0.01 * fabs(best[ip + 1]));
      if (o.X) o.X[o0 + s] = (float)(0.01 * fabs(best[ip + 2]));
    }
  }
}

// ---- binning by scene count --------------------------------------------
__global__ void bin_count_kernel(const int32_t *offsets, int64_t npix, int32_t *counts,
                                 photic_outputs o, unsigned int *error) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const int k = offsets[p + 1] - offsets[p];
  if (k >= 1 && k <= kMaxScenes) {
    atomicAdd(&counts[k - 1], 1);
  } else {
    if (o.status) o.status[p] = PHOTIC_PX_INVALID;
    if (o.depth) o.depth[p] = 0.0f;
    if (o.depth_f64) o.depth_f64[p] = 0.0;
    if (o.evals) o.evals[p] = 0;
    atomicOr(error, PHOTIC_DEVERR_BAD_SCENES);
  }
}

__global__ void bin_scan_kernel(const int32_t *counts, int32_t *start, int32_t *fill) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    int32_t acc = 0;
    for (int k = 0; k < kMaxScenes; k++) {
      start[k] = acc;
      fill[k] = acc;
      acc += counts[k];
    }
  }
}

__global__ void bin_scatter_kernel(const int32_t *offsets, int64_t npix, int32_t *fill,
                                   int32_t *list) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const int k = offsets[p + 1] - offsets[p];
  if (k >= 1 && k <= kMaxScenes) {
    const int32_t pos = atomicAdd(&fill[k - 1], 1);
    list[pos] = (int32_t)p;
  }
}

template <int LAYOUT, int K, int NB>
cudaError_t launch_k(const JointArgs &a, int grid, cudaStream_t s) {
  joint_kernel<LAYOUT, K, NB><<<grid, 128, 0, s>>>(a);
  return cudaGetLastError();
}

// The per-k kernels, largest k (longest fits) first.  With a fork set each
// goes to its own stream after the binning and joins back into s, so the
// kernels run side by side and one kernel's ragged tail is filled by the
// others' blocks; inside a stream capture the fork becomes parallel branches
// of the graph.  Without one they run in order on s.
template <int LAYOUT, int NB>
cudaError_t launch_all_k(const JointArgs &a, int sms, int per_sm, cudaStream_t s,
                         const JointFork *f) {
  const int grid = sms * (per_sm > 0 ? per_sm : 4);
  typedef cudaError_t (*Launch)(const JointArgs &, int, cudaStream_t);
  const Launch fn[kMaxScenes] = {launch_k<LAYOUT, 1, NB>, launch_k<LAYOUT, 2, NB>,
                                 launch_k<LAYOUT, 3, NB>, launch_k<LAYOUT, 4, NB>,
                                 launch_k<LAYOUT, 5, NB>, launch_k<LAYOUT, 6, NB>,
                                 launch_k<LAYOUT, 7, NB>, launch_k<LAYOUT, 8, NB>};
  cudaError_t e;
  if (f && (e = cudaEventRecord(f->fork, s)) != cudaSuccess) return e;
  for (int k = kMaxScenes; k >= 1; k--) {
    cudaStream_t t = f ? f->side[k - 1] : s;
    if (f && (e = cudaStreamWaitEvent(t, f->fork, 0)) != cudaSuccess) return e;
    // up to four bands: a group of lanes per pixel (photic_joint_group.cu);
    // more bands: one thread per pixel
    e = NB <= 4 ? launch_joint_group(a, k, per_sm, sms, t) : fn[k - 1](a, grid, t);
    if (e != cudaSuccess) return e;
    if (f) {
      if ((e = cudaEventRecord(f->join[k - 1], t)) != cudaSuccess) return e;
      if ((e = cudaStreamWaitEvent(s, f->join[k - 1], 0)) != cudaSuccess) return e;
    }
  }
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_joint(const JointArgs &a, int32_t *fill, int sms, int per_sm, cudaStream_t s,
                         const JointFork *f) {
  const int block = 256;
  const unsigned g = (unsigned)((a.npix + block - 1) / block);
  if (a.npix > 0) {
    bin_count_kernel<<<g, block, 0, s>>>(a.offsets, a.npix, a.bin_count, a.out, a.error);
    bin_scan_kernel<<<1, 32, 0, s>>>(a.bin_count, a.bin_start, fill);
    bin_scatter_kernel<<<g, block, 0, s>>>(a.offsets, a.npix, fill, a.list);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (a.fp.n_bands <= 4) {
    return a.fp.layout == PHOTIC_LAYOUT_REFERENCE ? launch_all_k<PHOTIC_LAYOUT_REFERENCE, 4>(a, sms, per_sm, s, f)
                                                  : launch_all_k<PHOTIC_LAYOUT_SCENE_B, 4>(a, sms, per_sm, s, f);
  }
  return a.fp.layout == PHOTIC_LAYOUT_REFERENCE ? launch_all_k<PHOTIC_LAYOUT_REFERENCE, 8>(a, sms, per_sm, s, f)
                                                : launch_all_k<PHOTIC_LAYOUT_SCENE_B, 8>(a, sms, per_sm, s, f);
}

}  // namespace photic
