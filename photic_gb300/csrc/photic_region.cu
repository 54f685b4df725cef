// photic_region.cu -- the general single-scene fit of samodel_optimise
// (model/samodel.c:1768-2115): each pixel alone (n_spatial = 1) or together
// with its 3 x 3 neighbourhood (n_spatial = 2; model/samodel.c:2957-3027:
// row and column indexes clamped at the grid's edges, neighbours with a
// nodata band left out, the centre's slot is the origin), with n_bottoms
// bottom types mixed per region (sand, seagrass, coral: the first entries of
// the reference's bottom table, all fitted at once as ALL_BOTTOMS selects,
// model/samodel.c:1822-1858).  Every region has its own depth and, per
// bottom type, its own albedo and mixing weight q; the scene's P, G, X are
// shared; the cost adds the depth- and bottom-continuity terms
// (model/samodel.c:2594-2692) to the spectral and K terms, and the depth
// reported is the origin-weighted mean (model/samodel.c:1999-2017).  A pixel
// with an empirical depth starts there alone, and one deeper than 8 m is
// fitted with sand alone (model/samodel.c:1781, 1826-1830, 2208-2231).
//
// Several scenes of the same place (own sun zenith, the same bands) are
// fitted jointly: every scene has its own P, G, X (model/samodel.c:
// 2463-2491).  One warp per pixel.  With R regions (1..9), Nb bottom types
// (1..3) and S scenes the simplex has n = R + 2 Nb R + 3 S <= 96
// coordinates, C per lane (the run-time-size NmGroup of photic_nmgroup.cuh),
// and the R * S * n_bands <= 128 band terms are spread over the lanes (lane
// l takes terms l, l + 32, l + 64, l + 96).  The lane at the head of the
// warp forms the cost from the terms in the reference's order (region,
// scene, band) and adds the continuity and K terms.  IEEE double in the
// reference's operation order throughout.
//
// Inputs come from a grid (the pixel loop of samodel()) or, for the
// per-pixel drop-ins, as explicit region lists (a model_data's regions);
// the list mode can also evaluate the cost at given parameters
// (samodel_error) instead of fitting.
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_fp64.cuh"
#include "photic_kernels.h"
#include "photic_nmgroup.cuh"

namespace photic {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxR = kRegionMaxR, kTerms = 128, kHT = kTerms / 32, kShares = 32, kRS = 64;

// Launch shapes: C coordinates per lane, vertex row stride CG.
template <int C, int CG>
struct Shape {
  static constexpr int kMaxN = C == 1 ? 32 : CG;
  static constexpr int kNF = kMaxN + 2;
  // doubles of shared memory per warp: vertices (n+1) x CG, per-lane vertex
  // costs, the evaluation point, band terms (residual^2, K, bottom share of
  // the reflectance), per-region Rrs(490/550/640), final details and
  // per-(region, bottom) shares of the bottom-continuity term
  static constexpr int kSmem =
      (kMaxN + 1) * CG + kNF * 32 + 32 * C + 3 * kTerms + 3 * kRS + 8 + kShares;
};

__device__ __forceinline__ bool nodata_value(float v, float nodata) {
  const float diff = __fsub_rn(v, nodata);
  const double big =
      fabs((double)v) < fabs((double)nodata) ? fabs((double)nodata) : fabs((double)v);
  return fabs((double)diff) <= big * (double)1.0e-6f;
}

// The regions of pixel p in the reference's order: their spectrum indexes
// (scene s of region r is row rp[r] * S + s of the list, or pixel rp[r] of
// scene s's grid), their count and the origin's slot.  A neighbour with a
// nodata band in any scene is left out.
__device__ __forceinline__ int regions_of(const RegionArgs &a, int64_t p, int64_t (&rp)[kMaxR],
                                          int &origin) {
  const int nb = a.fp.n_bands;
  if (a.list_R) {
    const int R = a.list_R[p];
    origin = a.list_origin[p];
    for (int r = 0; r < kMaxR; r++) rp[r] = p * kMaxR + (r < R ? r : 0);
    return R;
  }
  const int i = (int)(p / a.ncols), j = (int)(p % a.ncols);
  const int w = a.n_spatial - 1;
  int R = 0;
  origin = 0;
  for (int ii = -w; ii <= w; ii++) {
    const int iii = i + ii < 0 ? 0 : (i + ii > a.nrows - 1 ? a.nrows - 1 : i + ii);
    for (int jj = -w; jj <= w; jj++) {
      const int jjj = j + jj < 0 ? 0 : (j + jj > a.ncols - 1 ? a.ncols - 1 : j + jj);
      const int64_t q = (int64_t)iii * a.ncols + jjj;
      bool nodata = false;
      for (int s = 0; s < a.n_scenes; s++)
        for (int b = 0; b < nb; b++)
          if (nodata_value(a.grid[(s * a.npix + q) * nb + b], a.fp.nodata)) nodata = true;
      if (i == iii && j == jjj) origin = R;
      if (!nodata) rp[R++] = q;
    }
  }
  return R;
}

__device__ __forceinline__ void write_masked(const photic_outputs &o, int64_t p, int S,
                                             int32_t status) {
  if (o.depth) o.depth[p] = 0.0f;
  if (o.depth_f64) o.depth_f64[p] = 0.0;
  for (int s = 0; s < S; s++) {
    if (o.P) o.P[p * S + s] = 0.0f;
    if (o.G) o.G[p * S + s] = 0.0f;
    if (o.X) o.X[p * S + s] = 0.0f;
  }
  if (o.bottom_albedo) o.bottom_albedo[p] = 0.0f;
  if (o.model_error) o.model_error[p] = 0.0f;
  if (o.rrs_error) o.rrs_error[p] = 0.0f;
  if (o.K_min) o.K_min[p] = 0.0f;
  if (o.iod) o.iod[p] = 0.0f;
  if (o.evals) o.evals[p] = 0;
  if (o.evals_kept) o.evals_kept[p] = 0;
  if (o.status) o.status[p] = status;
  if (o.bottom_percent)
    for (int k = 0; k < 3; k++) o.bottom_percent[p * 3 + k] = 0.0f;
  if (o.bottom_type) o.bottom_type[p] = 0.0f;
}

template <int C, int CG, int BLOCK>
__global__ void __launch_bounds__(BLOCK) region_kernel(const __grid_constant__ RegionArgs a) {
  using Sh = Shape<C, CG>;
  constexpr int kMaxN = Sh::kMaxN, kNF = Sh::kNF;
  extern __shared__ double smem[];
  const FitParams &fp = a.fp;
  const SceneConsts &sc = a.sc;
  const photic_outputs &o = a.out;
  const int nb = fp.n_bands, S = a.n_scenes;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double *base = smem + warp * Sh::kSmem;
  double *V = base, *Fb = V + (kMaxN + 1) * CG, *X = Fb + kNF * 32, *dd = X + 32 * C,
         *kk = dd + kTerms, *io = kk + kTerms, *s490 = io + kTerms, *s550 = s490 + kRS,
         *s640 = s550 + kRS, *misc = s640 + kRS;
  double *share = misc + 8;
  const bool list = a.list_R != nullptr;
  // spectrum of scene s of region slot q (a pixel index of the grid, or a
  // region row of the list)
  auto spec = [&](int64_t q, int s) -> const float * {
    return list ? a.list_rrs + (q * S + s) * nb : a.grid + ((int64_t)s * a.npix + q) * nb;
  };

  NmGroup<0, C, 32, CG> m;
  m.V = V;
  m.Fv = Fb + lane;
  m.X = X;
  m.gl = lane;
  m.gmask = kFull;
  m.clear();
  m.nrt = 6;

  const double early = fp.early_exit_per_scene * (double)(float)S;

  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(a.queue, 1ull);
    t = __shfl_sync(kFull, t, 0);
    if (t >= (unsigned long long)a.npix) break;
    const int64_t p = (int64_t)t;

    // the pixel loop's mask test on the centre, every scene
    // (model/samodel.c:933-947); samodel_optimise called directly has none
    if (!a.no_mask) {
      bool masked = false;
      for (int s = 0; s < S; s++)
        for (int b = 0; b < nb; b++) {
          const float v = spec(p, s)[b];
          if (nodata_value(v, fp.nodata) || v < 0.0f) masked = true;
        }
      if (masked) {
        if (lane == 0) write_masked(o, p, S, PHOTIC_PX_MASKED);
        continue;
      }
    }

    // ---- set-up: regions, bottom types, per-term inputs
    int64_t rp[kMaxR];
    int origin = 0;
    const int R = regions_of(a, p, rp, origin);
    int nbt = a.n_bottoms;
    double hemp = __longlong_as_double(0x7ff8000000000000LL);
    if (a.h_emp) {
      hemp = a.h_emp[p];
      if (!isnan(hemp) && hemp > 8.0) nbt = 1;  // model/samodel.c:1781, 1826-1830
    }
    const int N = R + 2 * nbt * R + 3 * S, nterm = R * S * nb;
    const int qo = R + R * nbt, off = R + 2 * nbt * R;
    if (R < 1 || N > kMaxN || nterm > kTerms || R * S > kRS) {
      if (lane == 0) {
        atomicOr(a.error, PHOTIC_DEVERR_EVAL_CAP);
        write_masked(o, p, S, PHOTIC_PX_INVALID);
      }
      continue;
    }
    m.nrt = N;
    // term tau = ((r S + s) nb + b): region r, scene s, band b, in the order
    // samodel_error sums them (model/samodel.c:2465-2571)
    double my_rrs[kHT], my_pw[kHT], my_sec[kHT];
    int my_r[kHT], my_s[kHT], my_b[kHT];
    bool my_on[kHT];
#pragma unroll
    for (int h = 0; h < kHT; h++) {
      const int tau = lane + 32 * h;
      my_rrs[h] = my_pw[h] = my_sec[h] = 0.0;
      my_r[h] = my_s[h] = my_b[h] = 0;
      my_on[h] = tau < nterm;
      if (my_on[h]) {
        const int rs = tau / nb, b = tau % nb, r = rs / S, s = rs % S;
        const float *sp = spec(rp[r], s);
        double r8[kMaxBands];
#pragma unroll
        for (int c = 0; c < kMaxBands; c++) r8[c] = c < nb ? (double)sp[c] : 0.0;
        double r440 = interp_plan<kMaxBands>(fp.plan[0], r8);
        const double r490 = interp_plan<kMaxBands>(fp.plan[1], r8);
        if (r440 < 0.0) r440 = 0.0001;
        const double chi = r440 / r490;
        double Y = 3.44 * (1.0 - 3.17 * fm::exp_t(-2.01 * chi));
        if (Y < 0.0) Y = 0.0;
        if (Y > 2.5) Y = 2.5;
        my_rrs[h] = (double)sp[b];
        my_pw[h] = pow(sc.ratio440[b], Y);
        my_sec[h] = a.sec_sun[s];
        my_r[h] = r;
        my_s[h] = s;
        my_b[h] = b;
      }
    }
    for (int rs = lane; rs < R * S; rs += 32) {
      const float *sp = spec(rp[rs / S], rs % S);
      double r8[kMaxBands];
#pragma unroll
      for (int c = 0; c < kMaxBands; c++) r8[c] = c < nb ? (double)sp[c] : 0.0;
      s490[rs] = interp_plan<kMaxBands>(fp.plan[1], r8);
      s550[rs] = interp_plan<kMaxBands>(fp.plan[2], r8);
      s640[rs] = interp_plan<kMaxBands>(fp.plan[3], r8);
    }
    __syncwarp();
    // mean measured Rrs over all region-scene-bands, in the cost's order
    double tot = 0.0;
    if (lane == 0) {
      for (int r = 0; r < R; r++)
        for (int s = 0; s < S; s++)
          for (int b = 0; b < nb; b++) tot = tot + (double)spec(rp[r], s)[b];
    }
    tot = __shfl_sync(kFull, tot, 0);
    const double mean = tot / (double)nterm;

    // cold start of the lane's coordinates (model/samodel.c:2249-2353)
    auto cold = [&](double hs) {
#pragma unroll
      for (int tt = 0; tt < C; tt++) {
        const int c = lane + 32 * tt;
        double st = 0.0, sp = 0.0;
        if (c < R) {
          st = hs;
          sp = 1.25 * st;
        } else if (c < qo) {
          double m490 = 0.0;
          for (int rs = 0; rs < R * S; rs++) m490 += s490[rs];
          m490 /= (double)R * S;
          st = 100.0 * 4.0 * m490;
          sp = 1.5 * st;
        } else if (c < off) {
          st = 1.0;
          sp = 0.5 * st;
        } else if (c < N) {
          const int s = (c - off) / 3, j = (c - off) % 3;
          double m490 = 0.0, m550 = 0.0, m640 = 0.0;
          for (int r = 0; r < R; r++) {
            m490 += s490[r * S + s];
            m550 += s550[r * S + s];
            m640 += s640[r * S + s];
          }
          m490 /= (double)R;
          m550 /= (double)R;
          m640 /= (double)R;
          const double P = 100.0 * 0.072 * pow(m490 / m550, -1.7);
          st = j == 0 ? P : j == 1 ? 1.5 * P : 100.0 * 30.0 * fp.aw640 * m640;
          sp = 2.0 * st;
        }
        m.start[tt] = st;
        m.step[tt] = sp;
      }
    };

    const bool eval_only = a.eval_params != nullptr;
    const int n_starts = eval_only ? 0 : (isnan(hemp) ? fp.n_hstarts : 1);
    const double var_limit = fp.reqmin * (double)N;
    const int32_t guard_cap = (n_starts + 1) * (fp.kcount + 8 * N + 16);
    int32_t kst = 0, total = 0, kept_evals = 0, kept_start = 0, kept_fault = 0, guard = 0;
    double lowest = 1.0e4, best[C];
#pragma unroll
    for (int tt = 0; tt < C; tt++) best[tt] = 0.0;
    bool final_eval = eval_only;
    if (eval_only) {
      for (int c = lane; c < N; c += 32) X[c] = a.eval_params[p * a.eval_stride + c];
    } else {
      cold(isnan(hemp) ? fp.hstarts[0] : hemp);
      m.begin(var_limit, fp.konvge, fp.kcount);
    }

    for (;;) {
      __syncwarp();
      // ---- band terms at X
#pragma unroll
      for (int h = 0; h < kHT; h++) {
        if (!my_on[h]) continue;
        const int r = my_r[h], s = my_s[h], b = my_b[h], tau = lane + 32 * h;
        const double H = fabs(X[r]);
        const double P = 0.01 * fabs(X[off + 3 * s]);
        const double Gg = 0.01 * fabs(X[off + 1 + 3 * s]);
        const double Xx = 0.01 * fabs(X[off + 2 + 3 * s]);
        // bottom mixture of the region (model/samodel.c:2475-2496, 2878-2883);
        // the loops over the (at most 3) types are unrolled so the values
        // stay in registers
        double Bk[3], qk[3], q_sum = 0.0, rho = 0.0;
#pragma unroll
        for (int k = 0; k < 3; k++) {
          Bk[k] = k < nbt ? 0.01 * fabs(X[R + r * nbt + k]) : 0.0;
          qk[k] = k < nbt ? fabs(X[qo + r * nbt + k]) : 0.0;
        }
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (k < nbt) q_sum += qk[k];
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (k < nbt) qk[k] /= q_sum;
#pragma unroll
        for (int k = 0; k < 3; k++)
          if (k < nbt) rho += qk[k] * Bk[k] * sc.refl_k[k][b];
        const double lnP = log(P);
        const double a_phi = (sc.a0[b] + sc.a1[b] * lnP) * P;
        const double a_g = Gg * sc.eS[b];
        const double aa = sc.aw[b] + a_phi + a_g;
        const double bbk = sc.bbw[b] + Xx * my_pw[h];
        const double u = bbk / (aa + bbk);
        double Kb = aa + bbk;
        if (Kb < 0.0) Kb = 0.0;
        if (Kb > 2.5) Kb = 2.5;
        const double rrs_dp = (0.084 + 0.170 * u) * u;
        const double DuC = 1.03 * sqrt(1.0 + 2.4 * u);
        const double DuB = 1.04 * sqrt(1.0 + 5.4 * u);
        double M = my_sec[h] + DuC * sc.sec_view;
        const double rrs_C = rrs_dp * (1.0 - fm::exp_t(-M * Kb * H));
        M = my_sec[h] + DuB * sc.sec_view;
        const double rrs_B = fm::div_by(rho, kPi, fm::kInvPi) * fm::exp_t(-M * Kb * H);
        const double rrs = rrs_C + rrs_B;
        const double Rm = 0.5 * rrs / (1.0 - 1.5 * rrs);
        const double d = Rm - my_rrs[h];
        dd[tau] = d * d;
        kk[tau] = Kb;
        if (final_eval) {
          io[tau] = rrs_B / rrs;
          if (eval_only && a.eval_rm) a.eval_rm[((p * kMaxR + r) * S + s) * nb + b] = Rm;
        }
      }
      // each (region, bottom) share |100 B| |q| / sum |q| on its own lane
      // (the division is the costly part of the bottom-continuity term)
      if (lane < R * nbt) {
        const int r = lane / nbt, k = lane % nbt;
        double qs = 0.0;
        for (int kb = 0; kb < nbt; kb++) qs += fabs(X[qo + r * nbt + kb]);
        share[lane] = fabs(X[R + r * nbt + k]) * fabs(X[qo + r * nbt + k]) / qs;
      }
      __syncwarp();
      // ---- the cost on the head lane (model/samodel.c:2432-2759)
      double y = 0.0;
      if (lane == 0) {
        double err = 0.0;
        for (int tau = 0; tau < nterm; tau++) err = err + dd[tau];
        const double E = 100.0 * sqrt(fm::div_count(err, nterm)) / mean;
        // depth continuity
        double dmean = 0.0;
        for (int r = 0; r < R; r++) dmean += fabs(X[r]);
        dmean /= (double)R;
        double th = dmean < 4.0 ? 0.4 : dmean < 8.0 ? 0.2 : dmean < 12.0 ? 0.1 : 0.05;
        double Ed = 0.0, nout = 0.0;
        for (int r = 0; r < R; r++) {
          const double h = fabs(X[r]);
          if (h < (1.0 - th) * dmean || h > (1.0 + th) * dmean) {
            const double dv = h - dmean;
            Ed += dv * dv;
            nout += 1.0;
          }
        }
        if (nout > 0.5) Ed = 100.0 * sqrt(Ed / nout) / dmean;
        // bottom continuity, per bottom type
        th = dmean < 5.0 ? 0.25 : dmean < 10.0 ? 0.1 : dmean < 15.0 ? 0.05 : 0.01;
        double Eb = 0.0, btotal = 0.0;
        nout = 0.0;
        for (int k = 0; k < nbt; k++) {
          double bmean = 0.0;
          for (int r = 0; r < R; r++) bmean += share[r * nbt + k];
          bmean /= (double)R;
          btotal += bmean;
          for (int r = 0; r < R; r++) {
            const double bt = share[r * nbt + k];
            if (bt < (1.0 - th) * bmean || bt > (1.0 + th) * bmean) {
              const double dv = bt - bmean;
              Eb += dv * dv;
              nout += 1.0;
            }
          }
        }
        if (nout > 0.5) {
          const double bmean = btotal / ((double)nbt);
          Eb = 100.0 * sqrt(Eb / nout) / bmean;
        }
        // K terms: the origin's depth and each scene's K (the last region's
        // bands); the very-high-K term on the last scene's
        double km = 1.0e4, Ke = 0.0;
        const double Ho = fabs(X[origin]);
        for (int s = 0; s < S; s++) {
          km = 1.0e4;
          for (int b = 0; b < nb; b++) {
            const double Kb = kk[((R - 1) * S + s) * nb + b];
            if (__double2float_rn(Kb) != 0.0f && Kb < km) km = Kb;
          }
          Ke = Ke + k_penalty_f64(fp.kp, Ho, km);
        }
        if (km > 0.7) {
          const double dk = 4.0 * (km - 0.7);
          Ke = Ke + 100.0 * (dk * dk);
        }
        double model = 80.0 * E + 15.0 * Ed + 10.0 * Eb + 15.0 * Ke;
        model = fm::div_by(model, 120.0, fm::kInv120);
        y = model;
        if (final_eval) {
          double iod = 0.0, Kall = 1.0e4;
          for (int s = 0; s < S; s++)  // model/samodel.c:2051-2064
            for (int r = 0; r < R; r++)
              for (int b = 0; b < nb; b++) iod = iod + io[(r * S + s) * nb + b];
          for (int s = 0; s < S; s++)  // min over md->K, model/samodel.c:1994
            for (int b = 0; b < nb; b++) {
              const double Kb = kk[((R - 1) * S + s) * nb + b];
              if (__double2float_rn(Kb) != 0.0f && Kb < Kall) Kall = Kb;
            }
          // bottom albedo of the last region, sum_k q_k B_k (model/samodel.c:2878-2881)
          double qs = 0.0, alb = 0.0;
          for (int k = 0; k < nbt; k++) qs += fabs(X[qo + (R - 1) * nbt + k]);
          for (int k = 0; k < nbt; k++)
            alb += (fabs(X[qo + (R - 1) * nbt + k]) / qs) * (0.01 * fabs(X[R + (R - 1) * nbt + k]));
          misc[0] = E;
          misc[1] = model;
          misc[2] = alb;
          misc[3] = Kall == 1.0e4 ? 0.0 : Kall;
          misc[4] = 100.0 * iod / (double)nterm;
          misc[5] = km;
        }
      }
      y = __shfl_sync(kFull, y, 0);
      __syncwarp();

      if (eval_only) {
        if (lane == 0) {
          if (a.eval_cost) a.eval_cost[p] = y;
          if (a.eval_det) {
            a.eval_det[p * 8 + 0] = misc[0];
            a.eval_det[p * 8 + 1] = misc[1];
            a.eval_det[p * 8 + 2] = misc[2];
            a.eval_det[p * 8 + 3] = misc[5];
            a.eval_det[p * 8 + 4] = misc[4];
            a.eval_det[p * 8 + 5] = misc[3];
          }
        }
        break;
      }
      if (final_eval) {
        if (lane == 0) {
          const double ow = sqrt((double)R);
          double depth = 0.0;
          for (int r = 0; r < R; r++) {
            const double h = fabs(X[r]);
            if (r == origin) depth += ow * h;
            else depth += h;
          }
          depth /= ow + ((double)R) - 1.0;
          // bottom shares of the origin region and the bottom type
          // (model/samodel.c:2021-2047)
          double qs = 0.0, pct[3] = {0.0, 0.0, 0.0}, largest = 0.0, type = 0.0;
#pragma unroll
          for (int k = 0; k < 3; k++)
            if (k < nbt) qs += fabs(X[qo + origin * nbt + k]);
#pragma unroll
          for (int k = 0; k < 3; k++)
            if (k < nbt) pct[k] = 100.0 * fabs(X[qo + origin * nbt + k]) / qs;
#pragma unroll
          for (int k = 0; k < 3; k++)
            if (k < nbt && pct[k] > largest) {
              largest = pct[k];
              type = 1.0 + k;
            }
          if (o.depth) o.depth[p] = (float)depth;
          if (o.depth_f64) o.depth_f64[p] = depth;
          for (int s = 0; s < S; s++) {
            if (o.P) o.P[p * S + s] = (float)(0.01 * fabs(X[off + 3 * s]));
            if (o.G) o.G[p * S + s] = (float)(0.01 * fabs(X[off + 1 + 3 * s]));
            if (o.X) o.X[p * S + s] = (float)(0.01 * fabs(X[off + 2 + 3 * s]));
          }
          if (o.bottom_albedo) o.bottom_albedo[p] = (float)misc[2];
          if (o.model_error) o.model_error[p] = (float)misc[1];
          if (o.rrs_error) o.rrs_error[p] = (float)misc[0];
          if (o.K_min) o.K_min[p] = (float)misc[3];
          if (o.iod) o.iod[p] = (float)misc[4];
          if (o.evals) o.evals[p] = total;
          if (o.evals_kept) o.evals_kept[p] = kept_evals;
          if (o.bottom_percent)
            for (int k = 0; k < 3; k++) o.bottom_percent[p * 3 + k] = (float)pct[k];
          if (o.bottom_type) o.bottom_type[p] = (float)type;
          if (o.status)
            o.status[p] = PHOTIC_PX_FITTED | (kept_fault == 0 ? PHOTIC_PX_CONVERGED : 0) |
                          (kept_start << 16) | (R << 24);
        }
        if (a.list_params)
          for (int c = lane; c < N; c += 32) a.list_params[p * a.eval_stride + c] = X[c];
        break;
      }
      if (++guard > guard_cap) {
        if (lane == 0) {
          atomicOr(a.error, PHOTIC_DEVERR_EVAL_CAP);
          if (o.status) o.status[p] = PHOTIC_PX_INVALID;
        }
        break;
      }
      if (m.step_machine(y)) {
        // nelmin returned: keep the best start (model/samodel.c:2380-2405)
        const double ynewlo = m.F(m.lo);
        total += m.icount;
        bool finish = false;
        if (ynewlo < lowest) {
          lowest = ynewlo;
#pragma unroll
          for (int tt = 0; tt < C; tt++) best[tt] = m.xmin[tt];
          kept_evals = m.icount;
          kept_start = kst;
          kept_fault = m.ifault;
          if (lowest < early) finish = true;  // model/samodel.c:2404
        }
        kst++;
        if (finish || kst >= n_starts) {
#pragma unroll
          for (int tt = 0; tt < C; tt++)
            if (m.own(tt)) X[m.coord(tt)] = best[tt];  // re-evaluate at the kept optimum (:2413)
          final_eval = true;
        } else {
          double hs = fp.hstarts[0];
          for (int k = 1; k < kMaxHStarts; k++)
            if (k == kst) hs = fp.hstarts[k];
          cold(hs);
          m.begin(var_limit, fp.konvge, fp.kcount);
        }
      }
    }
    __syncwarp();
  }
}

template <int C, int CG, int BLOCK>
cudaError_t launch_shape(const RegionArgs &a, int sms, int per_sm, cudaStream_t s) {
  const size_t bytes = (size_t)(BLOCK / 32) * Shape<C, CG>::kSmem * sizeof(double);
  auto k = region_kernel<C, CG, BLOCK>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k, BLOCK, bytes);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  const int use = per_sm > 0 && per_sm < occ ? per_sm : occ;
  int64_t grid = (int64_t)sms * use;
  const int64_t need = (a.npix + BLOCK / 32 - 1) / (BLOCK / 32);
  if (grid > need) grid = need;
  k<<<(int)grid, BLOCK, bytes, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

int region_max_params(int max_regions, int n_bottoms, int n_scenes) {
  return max_regions + 2 * n_bottoms * max_regions + 3 * n_scenes;
}

cudaError_t launch_region(const RegionArgs &a, int max_params, int sms, int per_sm,
                          cudaStream_t s) {
  if (max_params <= Shape<1, 32>::kMaxN) return launch_shape<1, 32, 128>(a, sms, per_sm, s);
  if (max_params <= Shape<3, kRegionMaxParams>::kMaxN)
    return launch_shape<3, kRegionMaxParams, 32>(a, sms, per_sm, s);
  if (max_params <= Shape<3, 96>::kMaxN) return launch_shape<3, 96, 32>(a, sms, per_sm, s);
  return cudaErrorInvalidValue;
}

}  // namespace photic
