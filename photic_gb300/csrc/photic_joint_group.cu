// photic_joint_group.cu -- the temporal joint fit with a group of lanes per
// pixel.
//
// A pixel with k scenes has k x n_bands band terms per cost evaluation and
// a simplex of (n + 1) x n values, n = 3 + 3k or 1 + 4k.  One thread per
// pixel serialises all of it and keeps the simplex in local memory; here a
// group of G lanes (G = the power of two >= max(4k, n): 8, 16 or 32; 32 / G
// pixels per warp) shares the pixel:
//   * lane l evaluates band l % 4 of scene l / 4 (one band term per lane);
//     the lane at the head of the group then forms the cost from the terms
//     in the reference's order (scene, then band), so the sum rounds
//     exactly as samodel_error's does;
//   * the Nelder-Mead bookkeeping is split by coordinate: lane l owns
//     coordinate l (and l + 32 for the one n = 33 shape) of every vertex, centroid and
//     trial point, so the O(n^2) centroid becomes O(n) per lane; the
//     vertex costs (one copy per lane) and the decisions taken on them are
//     replicated in every lane of the group;
//   * vertices live in shared memory in lane-owned columns; the point to
//     evaluate is staged there for the band lanes.
// Every group reaches one cost evaluation per loop trip (the resumable
// state machine of photic_nm.cuh, restated per group), so the warp stays
// converged where the work is.  Arithmetic is IEEE double in the
// reference's operation order; the sequence of points, comparisons and
// counters is nelmin's (model/asa047.c:10-502) with the starts of
// model/samodel.c:2249-2353 and the cost of model/samodel.c:2432-2759 at
// n_scenes = k.
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_fp64.cuh"
#include "photic_kernels.h"
#include "photic_nm.cuh"
#include "photic_nmgroup.cuh"

namespace photic {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kBlock = 128;

template <int LAYOUT, int K>
struct JG {
  static constexpr int N = LAYOUT == PHOTIC_LAYOUT_REFERENCE ? 3 + 3 * K : 1 + 4 * K;
  // lanes per pixel: the power of two >= max(4k band terms, n coordinates),
  // at most a warp; only the n = 33 simplex (per-scene albedo, k = 8) gives
  // a lane two coordinates
  static constexpr int W = 4 * K > N ? 4 * K : N;
  static constexpr int G = W <= 4 ? 4 : W <= 8 ? 8 : W <= 16 ? 16 : 32;
  static constexpr int C = (N + G - 1) / G;   // coordinates per lane (<= 2)
  static_assert(C == 1 || G == 32, "a second coordinate slot only with a warp per pixel");
  static constexpr int CG = C * G;            // row length of a vertex
  static constexpr int NF = (N + 2) & ~1;     // vertex costs, padded
  // doubles of shared memory per group: vertices, per-lane vertex costs,
  // the evaluation point, band terms (squared residual, K, bottom share)
  // and the final cost details
  static constexpr int kSmem = (N + 1) * CG + NF * G + CG + 3 * G + 8 + 16;
  static constexpr int kGroups = kBlock / G;
};

// Per-group view of the shared memory.
struct GSmem {
  double *V, *F, *X, *dd, *kk, *io, *misc, *kmin, *kpen;
};

// Rrs(490), Rrs(550), Rrs(640) of scene s of the pixel whose observations
// start at o0 (model/samodel.c:1785-1793), read straight from the input.
// Each lane that needs them computes them itself: the start values depend
// on no other lane's shared-memory stores.
__device__ __forceinline__ void scene_shape(const JointArgs &a, int64_t o0, int s, double &r490,
                                            double &r550, double &r640) {
  const int nb = a.fp.n_bands;
  double r4[4];
#pragma unroll
  for (int b = 0; b < 4; b++) r4[b] = b < nb ? (double)a.rrs[(o0 + s) * nb + b] : 0.0;
  r490 = interp_plan<4>(a.fp.plan[1], r4);
  r550 = interp_plan<4>(a.fp.plan[2], r4);
  r640 = interp_plan<4>(a.fp.plan[3], r4);
}

// Cold start (model/samodel.c:2249-2353) for the lane's own coordinates;
// depth from hs.
template <int LAYOUT, int K, int N, int C, int G>
__device__ __forceinline__ void group_cold(const JointArgs &a, int64_t o0, int gl, double hs,
                                           double (&start)[C], double (&step)[C]) {
  const double c5 = 100.0 * 30.0 * a.fp.aw640;
#pragma unroll
  for (int t = 0; t < C; t++) {
    const int i = gl + t * G;
    double st = 0.0, sp = 0.0, r490 = 0.0, r550 = 0.0, r640 = 0.0;
    if (i >= N) {
      start[t] = 0.0;
      step[t] = 0.0;
      continue;
    }
    if (i == 0) {
      st = hs;
      sp = 1.25 * st;
    } else if (LAYOUT == PHOTIC_LAYOUT_REFERENCE) {
      if (i == 1) {
        double m490 = 0.0;
        for (int s = 0; s < K; s++) {
          scene_shape(a, o0, s, r490, r550, r640);
          m490 += r490;
        }
        m490 /= (double)1 * K;
        st = 100.0 * 4.0 * m490;
        sp = 1.5 * st;
      } else if (i == 2) {
        st = 1.0;
        sp = 0.5 * st;
      } else {
        const int s = (i - 3) / 3, r = (i - 3) % 3;
        scene_shape(a, o0, s, r490, r550, r640);
        const double P = 100.0 * 0.072 * pow(r490 / r550, -1.7);
        st = r == 0 ? P : r == 1 ? 1.5 * P : c5 * r640;
        sp = 2.0 * st;
      }
    } else {
      const int s = (i - 1) / 4, r = (i - 1) % 4;
      scene_shape(a, o0, s, r490, r550, r640);
      if (r == 0) {
        st = 100.0 * 4.0 * r490;
        sp = 1.5 * st;
      } else {
        const double P = 100.0 * 0.072 * pow(r490 / r550, -1.7);
        st = r == 1 ? P : r == 2 ? 1.5 * P : c5 * r640;
        sp = 2.0 * st;
      }
    }
    start[t] = st;
    step[t] = sp;
  }
}

template <int LAYOUT, int K>
__global__ void __launch_bounds__(kBlock) joint_group_kernel(const __grid_constant__ JointArgs a) {
  using D = JG<LAYOUT, K>;
  constexpr int N = D::N, G = D::G, C = D::C, CG = D::CG;
  extern __shared__ double smem[];
  const FitParams &fp = a.fp;
  const SceneConsts &sc = a.sc;
  const photic_outputs &o = a.out;
  const int nb = fp.n_bands;
  const int bin = K - 1;
  const int32_t count = a.bin_count[bin];
  const int32_t first = a.bin_start[bin];

  const int gid = threadIdx.x / G, gl = threadIdx.x % G;
  GSmem g;
  {
    double *base = smem + gid * D::kSmem;
    g.V = base;
    g.F = g.V + (N + 1) * CG;
    g.X = g.F + D::NF * G;
    g.dd = g.X + CG;
    g.kk = g.dd + G;
    g.io = g.kk + G;
    g.misc = g.io + G;
    g.kmin = g.misc + 8;
    g.kpen = g.kmin + 8;
  }
  NmGroup<N, C, G, CG> m;
  m.V = g.V;
  m.Fv = g.F + gl;
  m.X = g.X;
  m.gl = gl;
  m.clear();
  const unsigned gmask = (G == 32 ? kFull : ((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
  m.gmask = gmask;

  // the band this lane evaluates
  const int bs = gl >> 2, bb = gl & 3;
  const bool band_lane = bs < K && bb < nb;
  const int cB = LAYOUT == PHOTIC_LAYOUT_REFERENCE ? 1 : 1 + 4 * bs;
  const int cP = LAYOUT == PHOTIC_LAYOUT_REFERENCE ? 3 + 3 * bs : 2 + 4 * bs;

  const double var_limit = fp.reqmin * (double)N;
  const double early = fp.early_exit_per_scene * (double)(float)K;
  const int32_t guard_cap = (fp.n_hstarts + 1) * (fp.kcount + 8 * N + 16);

  bool has = false, exhausted = false, final_eval = false;
  int64_t p = 0, o0 = 0;
  int32_t kst = 0, total = 0, kept_evals = 0, kept_start = 0, kept_fault = 0, guard = 0;
  double lowest = 0.0, mean = 0.0;
  double best[C];
#pragma unroll
  for (int t = 0; t < C; t++) best[t] = 0.0;
  double my_rrs = 0.0, my_pw = 0.0, my_sec = 0.0;

  for (;;) {
    // ---- refill: a group without a pixel takes the next one of its bin
    unsigned long long tk = ~0ull;
    if (!has && !exhausted && gl == 0) tk = atomicAdd(&a.queues[bin], 1ull);
    tk = __shfl_sync(kFull, tk, 0, G);
    bool fresh = false;
    if (!has && !exhausted) {
      if (tk < (unsigned long long)count) {
        p = a.list[first + (int64_t)tk];
        o0 = a.offsets[p];
        fresh = true;
      } else {
        exhausted = true;
      }
    }
    if (__all_sync(kFull, !has && !fresh)) break;

    // ---- set-up of fresh pixels: per-band inputs, per-scene shape
    // values, mask test (model/samodel.c:933-947, 1785-1799)
    bool bad_band = false;
    if (fresh && band_lane) {
      const float rf = a.rrs[(o0 + bs) * nb + bb];
      const float diff = __fsub_rn(rf, fp.nodata);
      const double big = fabs((double)rf) < fabs((double)fp.nodata) ? fabs((double)fp.nodata)
                                                                    : fabs((double)rf);
      bad_band = fabs((double)diff) <= big * (double)1.0e-6f || rf < 0.0f;
      double r4[4];
#pragma unroll
      for (int b = 0; b < 4; b++) r4[b] = b < nb ? (double)a.rrs[(o0 + bs) * nb + b] : 0.0;
      my_rrs = r4[bb];
      double r440 = interp_plan<4>(fp.plan[0], r4);
      const double r490 = interp_plan<4>(fp.plan[1], r4);
      if (r440 < 0.0) r440 = 0.0001;
      const double chi = r440 / r490;
      double Y = 3.44 * (1.0 - 3.17 * fm::exp_t(-2.01 * chi));
      if (Y < 0.0) Y = 0.0;
      if (Y > 2.5) Y = 2.5;
      my_pw = pow(sc.ratio440[bb], Y);
      double th = a.theta_sun[o0 + bs];
      th *= 3.141592653589793 / 180.0;
      my_sec = 1.0 / cos(th);
      g.dd[gl] = my_rrs;
    }
    const bool masked = (__ballot_sync(kFull, bad_band) & gmask) != 0u;
    __syncwarp();
    double mtot = 0.0;
    if (fresh && gl == 0) {
      for (int s = 0; s < K; s++)
        for (int b = 0; b < nb; b++) mtot = mtot + g.dd[s * 4 + b];
      mtot = mtot / (double)(K * nb);
    }
    mtot = __shfl_sync(kFull, mtot, 0, G);
    if (fresh) {
      if (masked) {
        if (gl == 0) {
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
        }
        if (band_lane && bb == 0) {
          if (o.P) o.P[o0 + bs] = 0.0f;
          if (o.G) o.G[o0 + bs] = 0.0f;
          if (o.X) o.X[o0 + bs] = 0.0f;
        }
      } else {
        has = true;
        mean = mtot;
        total = kept_evals = kept_start = kept_fault = guard = 0;
        lowest = 1.0e4;
        final_eval = false;
#pragma unroll
        for (int t = 0; t < C; t++) best[t] = 0.0;
        kst = 0;
        group_cold<LAYOUT, K, N, C, G>(a, o0, gl, fp.hstarts[0], m.start, m.step);
        m.begin(var_limit, fp.konvge, fp.kcount);
      }
    }
    __syncwarp();

    // ---- one cost evaluation per group at X (model/samodel.c:2432-2759)
    if (has && band_lane) {
      const double *x = g.X;
      const double H = fabs(x[0]);
      double qB;
      if (LAYOUT == PHOTIC_LAYOUT_REFERENCE) {
        const double B = 0.01 * fabs(x[1]);
        const double qa = fabs(x[2]);
        qB = fm::self_ratio(qa) * B;
      } else {
        qB = 1.0 * (0.01 * fabs(x[cB]));
      }
      const double P = 0.01 * fabs(x[cP]);
      const double Gg = 0.01 * fabs(x[cP + 1]);
      const double Xx = 0.01 * fabs(x[cP + 2]);
      const double lnP = log(P);
      const double rho = qB * sc.refl[bb];
      const double a_phi = (sc.a0[bb] + sc.a1[bb] * lnP) * P;
      const double a_g = Gg * sc.eS[bb];
      const double aa = sc.aw[bb] + a_phi + a_g;
      const double bbk = sc.bbw[bb] + Xx * my_pw;
      const double u = bbk / (aa + bbk);
      double Kb = aa + bbk;
      if (Kb < 0.0) Kb = 0.0;
      if (Kb > 2.5) Kb = 2.5;
      const double rrs_dp = (0.084 + 0.170 * u) * u;
      const double DuC = 1.03 * sqrt(1.0 + 2.4 * u);
      const double DuB = 1.04 * sqrt(1.0 + 5.4 * u);
      double M = my_sec + DuC * sc.sec_view;
      const double rrs_C = rrs_dp * (1.0 - fm::exp_t(-M * Kb * H));
      M = my_sec + DuB * sc.sec_view;
      const double rrs_B = fm::div_by(rho, kPi, fm::kInvPi) * fm::exp_t(-M * Kb * H);
      const double rrs = rrs_C + rrs_B;
      const double Rm = 0.5 * rrs / (1.0 - 1.5 * rrs);
      const double d = Rm - my_rrs;
      g.dd[gl] = d * d;
      g.kk[gl] = Kb;
      if (final_eval) g.io[gl] = rrs_B / rrs;
    }
    __syncwarp();
    // each scene's K_min and K penalty on lane s (model/samodel.c:2696-2725);
    // only the sums that fix the rounding stay on the head lane
    if (has && gl < K) {
      const double H = fabs(g.X[0]);
      double km = 1.0e4;
      for (int b = 0; b < nb; b++) {
        const double Kb = g.kk[gl * 4 + b];
        if (__double2float_rn(Kb) != 0.0f && Kb < km) km = Kb;
      }
      g.kmin[gl] = km;
      g.kpen[gl] = k_penalty_f64(fp.kp, H, km);
    }
    __syncwarp();
    double y = 0.0;
    if (has && gl == 0) {
      double err = 0.0, Ke = 0.0, Kall = 1.0e4, iod = 0.0;
      for (int tau = 0; tau < K * 4; tau++)
        if ((tau & 3) < nb) err = err + g.dd[tau];
      for (int s = 0; s < K; s++) Ke = Ke + g.kpen[s];
      if (final_eval) {
        for (int s = 0; s < K; s++)
          for (int b = 0; b < nb; b++) {
            const double Kb = g.kk[s * 4 + b];
            iod = iod + g.io[s * 4 + b];
            if (__double2float_rn(Kb) != 0.0f && Kb < Kall) Kall = Kb;
          }
      }
      const double km = g.kmin[K - 1];
      const double E = 100.0 * sqrt(fm::div_count(err, K * nb)) / mean;
      if (km > 0.7) {  // the last scene's K_min (model/samodel.c:2726-2732)
        const double dk = 4.0 * (km - 0.7);
        Ke = Ke + 100.0 * (dk * dk);
      }
      double model = 80.0 * E + 15.0 * Ke;
      model = fm::div_by(model, 120.0, fm::kInv120);
      y = model;
      if (final_eval) {
        double qB;
        if (LAYOUT == PHOTIC_LAYOUT_REFERENCE) {
          const double B = 0.01 * fabs(g.X[1]);
          const double qa = fabs(g.X[2]);
          qB = fm::self_ratio(qa) * B;
        } else {
          qB = 1.0 * (0.01 * fabs(g.X[1 + 4 * (K - 1)]));
        }
        g.misc[0] = E;
        g.misc[1] = model;
        g.misc[2] = qB;
        g.misc[3] = Kall == 1.0e4 ? 0.0 : Kall;
        g.misc[4] = 100.0 * iod / (double)(K * nb);
      }
    }
    y = __shfl_sync(kFull, y, 0, G);
    __syncwarp();

    // ---- outputs of a finished pixel
    if (has && final_eval) {
      if (gl == 0) {
        const double H = fabs(g.X[0]);
        if (o.depth) o.depth[p] = (float)H;
        if (o.depth_f64) o.depth_f64[p] = H;
        if (o.bottom_albedo) o.bottom_albedo[p] = (float)g.misc[2];
        if (o.model_error) o.model_error[p] = (float)g.misc[1];
        if (o.rrs_error) o.rrs_error[p] = (float)g.misc[0];
        if (o.K_min) o.K_min[p] = (float)g.misc[3];
        if (o.iod) o.iod[p] = (float)g.misc[4];
        if (o.evals) o.evals[p] = total;
        if (o.evals_kept) o.evals_kept[p] = kept_evals;
        if (o.status)
          o.status[p] = PHOTIC_PX_FITTED | (kept_fault == 0 ? PHOTIC_PX_CONVERGED : 0) |
                        (kept_start << 16);
      }
      if (band_lane && bb == 0) {
        if (o.P) o.P[o0 + bs] = (float)(0.01 * fabs(g.X[cP]));
        if (o.G) o.G[o0 + bs] = (float)(0.01 * fabs(g.X[cP + 1]));
        if (o.X) o.X[o0 + bs] = (float)(0.01 * fabs(g.X[cP + 2]));
      }
      has = false;
      final_eval = false;
    } else if (has) {
      // ---- Nelder-Mead: consume y, stage the next point
      if (++guard > guard_cap) {
        // each nelmin call is bounded by kcount; reaching this is a defect
        if (gl == 0) {
          atomicOr(a.error, PHOTIC_DEVERR_EVAL_CAP);
          if (o.status) o.status[p] = PHOTIC_PX_INVALID;
        }
        has = false;
      } else if (m.step_machine(y)) {
        // nelmin returned: keep the best start (model/samodel.c:2380-2405)
        const double ynewlo = m.F(m.lo);
        total += m.icount;
        bool finish = false;
        if (ynewlo < lowest) {
          lowest = ynewlo;
#pragma unroll
          for (int t = 0; t < C; t++) best[t] = m.xmin[t];
          kept_evals = m.icount;
          kept_start = kst;
          kept_fault = m.ifault;
          if (lowest < early) finish = true;  // model/samodel.c:2404
        }
        kst++;
        if (finish || kst >= fp.n_hstarts) {
          m.set_x_from(best);  // re-evaluate at the kept optimum (:2413)
          final_eval = true;
        } else {
          double h = fp.hstarts[0];
          for (int i = 1; i < kMaxHStarts; i++)
            if (i == kst) h = fp.hstarts[i];
          group_cold<LAYOUT, K, N, C, G>(a, o0, gl, h, m.start, m.step);
          m.begin(var_limit, fp.konvge, fp.kcount);
        }
      }
    }
    __syncwarp();
  }
}

template <int LAYOUT, int K>
cudaError_t launch_group_k(const JointArgs &a, int per_sm, int sms, cudaStream_t s) {
  using D = JG<LAYOUT, K>;
  const size_t bytes = (size_t)D::kGroups * D::kSmem * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(joint_group_kernel<LAYOUT, K>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, joint_group_kernel<LAYOUT, K>, kBlock,
                                                    bytes);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  const int use = per_sm > 0 && per_sm < occ ? per_sm : occ;
  joint_group_kernel<LAYOUT, K><<<sms * use, kBlock, bytes, s>>>(a);
  return cudaGetLastError();
}

template <int LAYOUT>
cudaError_t launch_group_layout(const JointArgs &a, int k, int per_sm, int sms, cudaStream_t s) {
  switch (k) {
    case 1: return launch_group_k<LAYOUT, 1>(a, per_sm, sms, s);
    case 2: return launch_group_k<LAYOUT, 2>(a, per_sm, sms, s);
    case 3: return launch_group_k<LAYOUT, 3>(a, per_sm, sms, s);
    case 4: return launch_group_k<LAYOUT, 4>(a, per_sm, sms, s);
    case 5: return launch_group_k<LAYOUT, 5>(a, per_sm, sms, s);
    case 6: return launch_group_k<LAYOUT, 6>(a, per_sm, sms, s);
    case 7: return launch_group_k<LAYOUT, 7>(a, per_sm, sms, s);
    case 8: return launch_group_k<LAYOUT, 8>(a, per_sm, sms, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_joint_group(const JointArgs &a, int k, int per_sm, int sms, cudaStream_t s) {
  return a.fp.layout == PHOTIC_LAYOUT_REFERENCE
             ? launch_group_layout<PHOTIC_LAYOUT_REFERENCE>(a, k, per_sm, sms, s)
             : launch_group_layout<PHOTIC_LAYOUT_SCENE_B>(a, k, per_sm, sms, s);
}

}  // namespace photic
