// photic_invert.cu -- persistent, work-queue batched inversion of
// single-scene pixels (the plain method).
//
// One lane owns one pixel at a time and runs the whole per-pixel driver of
// samodel_optimise (model/samodel.c:1768-2115) with its cold depth starts
// and early exit (model/samodel.c:2243-2407) on the resumable Nelder-Mead
// of photic_nm.cuh.  Every loop trip all lanes that hold a pixel evaluate
// the cost together; when a lane's pixel is finished it takes the next one
// from its warp's chunk, and a warp whose chunk is used up claims the next
// 32 pixels with one atomic and stages their spectra through shared memory
// with coalesced (float4 when the layout allows) loads.  Ragged iteration
// counts (a few hundred to several thousand evaluations per pixel) thus
// never leave a lane idle while work remains.
//
// The arithmetic is a policy: PrecF64 (IEEE double, reference operation
// order, --fmad=false), PrecF32 (the forward model in float with the
// special-function unit, the simplex in double) or PrecDF (double-float on
// the FP32 pipes).
//
// Scratch: one 64-bit queue head per call (stream-ordered allocation in
// photic_host.cu) and the per-device sticky error word.
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_dfcost.cuh"
#include "photic_fp64.cuh"
#include "photic_kernels.h"
#include "photic_nm.cuh"
#include "photic_prec64.cuh"

namespace photic {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kN = 6;  // H, 100B, q, 100P, 100G, 100X

// ---------------------------------------------------------------------------
// Precision policies (PrecF64 is in photic_prec64.cuh)
// ---------------------------------------------------------------------------
// Single-precision forward model (FP32 with the special-function unit):
// the cost of a double parameter vector evaluated in float with the
// special-function unit's exp and log and approximate divisions, returned as
// a double; the simplex, its decisions, the convergence and local-minimum
// tests and the final re-evaluation at the kept optimum stay in FP64.
template <int NB>
struct PixelF32 {
  PixelF64<NB> d;        // the double set-up (cold starts, details)
  float rrs[NB], pw[NB];
  float mean;
};

struct PrecF32 : PrecF64 {
  static constexpr bool kFused = false;  // its products come from an FP64 evaluation
  template <int NB>
  using Pixel = PixelF32<NB>;
  template <int NB>
  static __device__ __forceinline__ void setup(const InvertArgs &a, const float *r, Pixel<NB> &px) {
    PrecF64::setup<NB>(a, r, px.d);
#pragma unroll
    for (int b = 0; b < NB; b++) {
      px.rrs[b] = (float)px.d.rrs[b];
      px.pw[b] = (float)px.d.pw[b];
    }
    px.mean = (float)px.d.mean;
  }
  template <int NB>
  static __device__ __forceinline__ void cold_start(const InvertArgs &a, const Pixel<NB> &px,
                                                    T *start, T *step) {
    cold_start_f64<NB>(a.fp, px.d, start, step);
  }
  // samodel_error (model/samodel.c:2432-2759) over samodel_Rrs (:2846-2949)
  // for one region, scene and bottom type, in float
  template <int NB>
  static __device__ __forceinline__ T cost(const InvertArgs &a, const Pixel<NB> &px, const T *x) {
    const FitParams &fp = a.fp;
    const SceneConsts &sc = a.sc;
    const int nb = fp.n_bands;
    const float H = fabsf((float)x[0]);
    const float B = 0.01f * fabsf((float)x[1]);
    const float qa = fabsf((float)x[2]);
    const float q = qa / qa;
    const float P = 0.01f * fabsf((float)x[3]);
    const float G = 0.01f * fabsf((float)x[4]);
    const float X = 0.01f * fabsf((float)x[5]);
    const float lnP = __logf(P);
    const float qB = q * B;
    const float ss = (float)sc.sec_sun, sv = (float)sc.sec_view;
    float err = 0.0f, K_min = 1.0e4f;
#pragma unroll
    for (int b = 0; b < NB; b++) {
      if (b < nb) {
        const float rho = qB * (float)sc.refl[b];
        const float a_phi = ((float)sc.a0[b] + (float)sc.a1[b] * lnP) * P;
        const float a_g = G * (float)sc.eS[b];
        const float aa = (float)sc.aw[b] + a_phi + a_g;
        const float bb = (float)sc.bbw[b] + X * px.pw[b];
        const float u = __fdividef(bb, aa + bb);
        float K = aa + bb;
        K = fminf(fmaxf(K, 0.0f), 2.5f);
        const float rrs_dp = (0.084f + 0.170f * u) * u;
        const float DuC = 1.03f * sqrtf(1.0f + 2.4f * u);
        const float DuB = 1.04f * sqrtf(1.0f + 5.4f * u);
        const float rrs_C = rrs_dp * (1.0f - __expf(-(ss + DuC * sv) * K * H));
        const float rrs_B = rho * 0.31830988618f * __expf(-(ss + DuB * sv) * K * H);
        const float rrs = rrs_C + rrs_B;
        const float Rm = __fdividef(0.5f * rrs, 1.0f - 1.5f * rrs);
        const float d = Rm - px.rrs[b];
        err += d * d;
        if (K != 0.0f && K < K_min) K_min = K;
      }
    }
    const float E = __fdividef(100.0f * sqrtf(err / (float)nb), px.mean);
    float Ke = 0.0f;
    int c = -1;
    const KPenalty &kp = fp.kp;
    if (H < 1.0f && K_min < (float)kp.k_thr[0]) c = 0;
    else if (H < 2.0f && K_min < (float)kp.k_thr[1]) c = 1;
    else if (H < 3.0f && K_min < (float)kp.k_thr[2]) c = 2;
    else if (H < 4.0f && K_min < (float)kp.k_thr[3]) c = 3;
    else if (H < 5.0f && K_min < (float)kp.k_thr[4]) c = 4;
    if (c >= 0) {
      float it = (float)kp.inv_t[0];
      for (int i = 1; i < 5; i++)
        if (i == c) it = (float)kp.inv_t[i];
      const float d = __fdividef(1.0f, 0.01f + K_min) - it;
      Ke = 100.0f * d * d;
    }
    if (K_min > 0.7f) {
      const float d = 4.0f * (K_min - 0.7f);
      Ke += 100.0f * d * d;
    }
    return (double)((80.0f * E + 15.0f * Ke) * (1.0f / 120.0f));
  }
  template <int NB>
  static __device__ __forceinline__ void details(const InvertArgs &a, const Pixel<NB> &px,
                                                 const T *x, Details &d) {
    PrecF64::details<NB>(a, px.d, x, d);
  }
};

struct PrecDF {
  static constexpr bool kFused = false;
  using T = df64;
  template <int NB>
  using Pixel = PixelDF<NB>;
  struct Details {
    double rrs_error, model_error, bottom_albedo, K_min, iod;
  };
  static __device__ __forceinline__ T zero() { return df64{0.0f, 0.0f}; }
  static __device__ __forceinline__ T one() { return df64{1.0f, 0.0f}; }
  static __device__ __forceinline__ T add(T a, T b) { return df_add(a, b); }
  static __device__ __forceinline__ T sub(T a, T b) { return df_sub(a, b); }
  static __device__ __forceinline__ T mul(T a, T b) { return df_mul(a, b); }
  static __device__ __forceinline__ T mul2(T a) { return df64{2.0f * a.hi, 2.0f * a.lo}; }
  static __device__ __forceinline__ T half(T a) { return df64{0.5f * a.hi, 0.5f * a.lo}; }
  static __device__ __forceinline__ T scale2(T a, float c) { return df64{c * a.hi, c * a.lo}; }
  static __device__ __forceinline__ T div_n(T a, int n) { return df_div_f(a, (float)n); }
  static __device__ __forceinline__ bool lt(T a, T b) { return df_lt(a, b); }
  static __device__ __forceinline__ bool le(T a, T b) { return df_le(a, b); }
  static __device__ __forceinline__ T eps_step(T s) { return df_mul(s, DFK(1.0e-6)); }
  static __device__ __forceinline__ T eps_scale() { return DFK(1.0e-6); }
  static __device__ __forceinline__ long long trunc10(T y) { return df_trunc10(y); }
  static __device__ __forceinline__ T from_double(double d) { return df_from_double(d); }
  static __device__ __forceinline__ double to_double(T a) { return df_to_double(a); }
  static __device__ __forceinline__ T var_limit(const InvertArgs &a) { return dp(a.ds.reqmin_n); }
  static __device__ __forceinline__ T hstart(const InvertArgs &a, int k) {
    DfPair h = a.ds.hstarts[0];
    for (int i = 1; i < kMaxHStarts; i++)
      if (i == k) h = a.ds.hstarts[i];
    return dp(h);
  }
  static __device__ __forceinline__ T h_step(T h) { return df_mul_f(h, 1.25f); }
  template <int NB>
  static __device__ __forceinline__ void setup(const InvertArgs &a, const float *r, Pixel<NB> &px) {
    pixel_setup_df<NB>(a.fp, a.ds, r, px);
  }
  template <int NB>
  static __device__ __forceinline__ void cold_start(const InvertArgs &a, const Pixel<NB> &px,
                                                    T *start, T *step) {
    cold_start_df<NB>(a.fp, a.ds, px, start, step);
  }
  template <int NB>
  static __device__ __forceinline__ T cost(const InvertArgs &a, const Pixel<NB> &px, const T *x) {
    return cost_df<false, NB>(a.fp, a.ds, px, x, nullptr);
  }
  template <int NB>
  static __device__ __forceinline__ void details(const InvertArgs &a, const Pixel<NB> &px,
                                                 const T *x, Details &d) {
    CostDetailsDF det;
    cost_df<true, NB>(a.fp, a.ds, px, x, &det);
    d.rrs_error = df_to_double(det.rrs_error);
    d.model_error = df_to_double(det.model_error);
    d.bottom_albedo = df_to_double(det.bottom_albedo);
    d.K_min = df_to_double(det.K_min);
    d.iod = df_to_double(det.iod);
  }
};

template <class P, int NB, int BS>
__global__ void __launch_bounds__(BS) invert_kernel(const __grid_constant__ InvertArgs args) {
  using T = typename P::T;
  const FitParams &fp = args.fp;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T *sv = reinterpret_cast<T *>(smem_raw);          // [(N+1)*N][BS]
  T *sf = sv + (kN + 1) * kN * BS;                  // [N+1][BS]
  T *sbest = sf + (kN + 1) * BS;                    // [N][BS]
  using Px = typename P::template Pixel<NB>;
  Px *spx = reinterpret_cast<Px *>(sbest + kN * BS);  // [BS/32][32] set-ups of the chunk
  float *schunk = reinterpret_cast<float *>(spx + BS);  // [BS/32][32][NB]

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float *wchunk = schunk + warp * 32 * NB;
  Px *wpx = spx + warp * 32;
  const unsigned lt_mask = (1u << lane) - 1u;

  NmLane<kN, P, BS> m;
  m.v = sv + tid;
  m.f = sf + tid;
  T *best = sbest + tid;
  typename P::template Pixel<NB> px;
  const T var_limit = P::var_limit(args);
  const photic_outputs &o = args.out;

  int64_t pixel = -1;
  int32_t start_k = 0, n_starts = 0, total = 0, kept_evals = 0, kept_start = 0, kept_fault = 0;
  int32_t guard = 0;
  T lowest = P::zero();

  bool has = false, open = true;
  int64_t chunk_base = 0, chunk_next = 0, chunk_end = 0;
  const int32_t guard_cap = (fp.n_hstarts + 1) * (fp.kcount + 8 * kN + 16);

  for (;;) {
    // ---- hand out pixels to lanes that have none -------------------------
    unsigned need = __ballot_sync(kFull, !has && open);
    while (need) {
      if (chunk_next >= chunk_end) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(args.queue, 32ull);
        base = __shfl_sync(kFull, base, 0);
        if (base >= (unsigned long long)args.npix) {
          open = false;
          break;
        }
        chunk_base = (int64_t)base;
        chunk_next = chunk_base;
        chunk_end = min(chunk_base + 32, args.npix);
        __syncwarp();
        const int64_t q = chunk_base + lane;
        if (q < args.npix) {
          const int64_t p = args.order ? (int64_t)args.order[q] : q;
          if (NB == 4 && args.vec4) {
            const float4 v4 = __ldg(reinterpret_cast<const float4 *>(args.rrs) + p);
            wchunk[lane * NB + 0] = v4.x;
            wchunk[lane * NB + 1] = v4.y;
            wchunk[lane * NB + 2] = v4.z;
            wchunk[lane * NB + 3] = v4.w;
          } else {
#pragma unroll
            for (int b = 0; b < NB; b++)
              wchunk[lane * NB + b] =
                  b < fp.n_bands ? __ldg(args.rrs + p * args.pixel_stride + b * args.band_stride)
                                 : 0.0f;
          }
          // every lane sets up one pixel of the chunk (interpolated Rrs,
          // Y and (440/lambda)^Y, model/samodel.c:1783-1799, 2897-2902)
          // with the whole warp, instead of each lane alone when it takes
          // the pixel; a masked pixel's set-up is never used
          float r[NB];
#pragma unroll
          for (int b = 0; b < NB; b++) r[b] = wchunk[lane * NB + b];
          P::template setup<NB>(args, r, wpx[lane]);
        }
        __syncwarp();
      }
      const int rank = __popc(need & lt_mask);
      const int avail = (int)(chunk_end - chunk_next);
      const bool mine = ((need >> lane) & 1u) && rank < avail;
      const unsigned taken = __ballot_sync(kFull, mine);
      bool masked = false;
      if (mine) {
        const int64_t q = chunk_next + rank;  // queue position -> pixel
        const int64_t p = args.order ? (int64_t)args.order[q] : q;
        float r[NB];
#pragma unroll
        for (int b = 0; b < NB; b++) r[b] = wchunk[(q - chunk_base) * NB + b];
#pragma unroll
        for (int b = 0; b < NB; b++)
          if (b < fp.n_bands && !args.no_mask && band_masked(r[b], fp.nodata)) masked = true;
        if (masked) {
          write_masked(o, p);
        } else {
          px = wpx[q - chunk_base];
          pixel = p;
          total = kept_evals = kept_start = kept_fault = guard = 0;
          lowest = P::from_double(1.0e4);
          start_k = 0;
          bool seeded = false;
#pragma unroll
          for (int i = 0; i < kN; i++) best[i * BS] = P::zero();
          if (args.seeds != nullptr) {
            const double *sd = args.seeds + p * kN;
            if (!isnan(sd[0])) {
              const double rel[kN] = {1.25, 1.5, 0.5, 2.0, 2.0, 2.0};
              seeded = true;
#pragma unroll
              for (int i = 0; i < kN; i++) {
                m.start[i] = P::from_double(sd[i]);
                m.step[i] = P::from_double((rel[i] * fp.seed_step_scale) * sd[i]);
              }
            }
          }
          n_starts = seeded ? 1 : fp.n_hstarts;
          if (!seeded) {
            P::template cold_start<NB>(args, px, m.start, m.step);
            m.start[0] = P::hstart(args, 0);
            m.step[0] = P::h_step(m.start[0]);
          }
          m.begin(var_limit, fp.konvge, fp.kcount);
          has = true;
        }
      }
      chunk_next += __popc(taken);
      need &= ~taken;
      need |= __ballot_sync(kFull, mine && masked);
    }
    if (!__any_sync(kFull, has)) break;

    // ---- one cost evaluation per lane, then the bookkeeping --------------
    if (has) {
      const bool fin = m.phase == PH_FINAL;
      typename P::Details det;
      T y = P::zero();
      if constexpr (P::kFused) {
        // the kept optimum is evaluated together with the other lanes' points
        typename P::template Keep<NB> keep;
        y = P::template cost_keep<NB>(args, px, m.x, keep);
        if (fin) P::template details_from_keep<NB>(args, keep, y, det);
      } else {
        if (fin) P::template details<NB>(args, px, m.x, det);
        else y = P::template cost<NB>(args, px, m.x);
      }
      if (fin) {
        const int64_t p = pixel;
        const double H = fabs(P::to_double(m.x[0]));
        if (o.depth) o.depth[p] = (float)H;
        if (o.depth_f64) o.depth_f64[p] = H;
        if (o.P) o.P[p] = (float)(0.01 * fabs(P::to_double(m.x[3])));
        if (o.G) o.G[p] = (float)(0.01 * fabs(P::to_double(m.x[4])));
        if (o.X) o.X[p] = (float)(0.01 * fabs(P::to_double(m.x[5])));
        if (o.bottom_albedo) o.bottom_albedo[p] = (float)det.bottom_albedo;
        if (o.model_error) o.model_error[p] = (float)det.model_error;
        if (o.rrs_error) o.rrs_error[p] = (float)det.rrs_error;
        if (o.K_min) o.K_min[p] = (float)det.K_min;
        if (o.iod) o.iod[p] = (float)det.iod;
        if (o.evals) o.evals[p] = total;
        if (o.evals_kept) o.evals_kept[p] = kept_evals;
        if (o.params)
          for (int i = 0; i < kN; i++) o.params[p * kN + i] = P::to_double(m.x[i]);
        if (o.status)
          o.status[p] = PHOTIC_PX_FITTED | (kept_fault == 0 ? PHOTIC_PX_CONVERGED : 0) |
                        (kept_start << 16);
        has = false;
      } else {
        if (++guard > guard_cap) {
          // Defensive cap: each nelmin call is bounded by kcount, so
          // reaching this means a defect; flag it instead of spinning.
          atomicOr(args.error, PHOTIC_DEVERR_EVAL_CAP);
          if (o.status) o.status[pixel] = PHOTIC_PX_INVALID;
          has = false;
        } else if (m.step_machine(y)) {
          // nelmin returned: keep the best start (model/samodel.c:2380-2405)
          const T ynewlo = m.F(m.lo);
          total += m.icount;
          bool finish = false;
          if (P::lt(ynewlo, lowest)) {
            lowest = ynewlo;
#pragma unroll
            for (int i = 0; i < kN; i++) best[i * BS] = m.xmin[i];
            kept_evals = m.icount;
            kept_start = start_k;
            kept_fault = m.ifault;
            if (P::lt(lowest, P::from_double(args.early_exit))) finish = true;
          }
          start_k++;
          if (!finish && start_k < n_starts) {
            P::template cold_start<NB>(args, px, m.start, m.step);
            m.start[0] = P::hstart(args, start_k);
            m.step[0] = P::h_step(m.start[0]);
            m.begin(var_limit, fp.konvge, fp.kcount);
          } else {
#pragma unroll
            for (int i = 0; i < kN; i++) m.x[i] = best[i * BS];
            m.phase = PH_FINAL;
          }
        }
      }
    }
  }
}

template <class P, int NB, int BS>
cudaError_t launch_one(const InvertArgs &a, int grid, cudaStream_t s, int *occupancy) {
  const size_t smem = invert_smem_bytes(BS, NB) + (size_t)BS * sizeof(typename P::template Pixel<NB>);
  auto k = invert_kernel<P, NB, BS>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (occupancy) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occupancy, k, BS, smem);
  k<<<grid, BS, smem, s>>>(a);
  return cudaGetLastError();
}

template <class P, int NB>
cudaError_t launch_block(const InvertArgs &a, int block, int grid, cudaStream_t s, int *occ) {
  switch (block) {
    case 64: return launch_one<P, NB, 64>(a, grid, s, occ);
    case 256: return launch_one<P, NB, 256>(a, grid, s, occ);
    default: return launch_one<P, NB, 128>(a, grid, s, occ);
  }
}

template <class P>
cudaError_t launch_prec(const InvertArgs &a, int block, int grid, cudaStream_t s, int *occ) {
  if (a.fp.n_bands == 4) return launch_block<P, 4>(a, block, grid, s, occ);
  return launch_block<P, 8>(a, block, grid, s, occ);
}

}  // namespace

// Shared memory of the simplex and the staged spectra; launch_one adds the
// chunk's pixel set-ups, whose size depends on the precision policy.
size_t invert_smem_bytes(int block, int nb) {
  // double and double-float both take 8 bytes per value
  return (size_t)block * 8 * ((kN + 1) * kN + (kN + 1) + kN) +
         (size_t)(block / 32) * 32 * (nb <= 4 ? 4 : 8) * sizeof(float);
}

cudaError_t launch_invert(const InvertArgs &a, int precision, int block, int grid,
                          cudaStream_t s) {
  if (precision == PHOTIC_PREC_DF64) return launch_prec<PrecDF>(a, block, grid, s, nullptr);
  if (precision == PHOTIC_PREC_FP32) return launch_prec<PrecF32>(a, block, grid, s, nullptr);
  return launch_prec<PrecF64>(a, block, grid, s, nullptr);
}

int invert_blocks_per_sm(const InvertArgs &a, int precision, int block) {
  int n = 0;
  cudaError_t e = precision == PHOTIC_PREC_DF64   ? launch_prec<PrecDF>(a, block, 0, 0, &n)
                  : precision == PHOTIC_PREC_FP32 ? launch_prec<PrecF32>(a, block, 0, 0, &n)
                                                  : launch_prec<PrecF64>(a, block, 0, 0, &n);
  return e == cudaSuccess ? n : 0;
}

}  // namespace photic
