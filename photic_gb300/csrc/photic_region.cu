// photic_region.cu -- the spatial-region fit (n_spatial = 2): each pixel is
// fitted together with its 3 x 3 neighbourhood (model/samodel.c:2957-3027:
// row and column indexes clamped at the grid's edges, neighbours with a
// nodata band left out, the centre's slot is the origin).  Every region has
// its own depth, albedo and q; the scene's P, G, X are shared; the cost adds
// the depth- and bottom-continuity terms (model/samodel.c:2594-2692) to the
// spectral and K terms, and the depth reported is the origin-weighted mean
// (model/samodel.c:1999-2017).  One scene, one bottom type.
//
// One warp per pixel.  With R regions (1..9) the simplex has n = 3R + 3 <= 30
// coordinates, one per lane (the run-time-size NmGroup of
// photic_nmgroup.cuh), and the R * n_bands <= 36 band terms are spread over
// the lanes (lane l takes terms l and l + 32).  The lane at the head of the
// warp forms the cost from the terms in the reference's order (region, then
// band) and adds the continuity and K terms.  IEEE double in the reference's
// operation order throughout.
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_fp64.cuh"
#include "photic_kernels.h"
#include "photic_nmgroup.cuh"

namespace photic {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kBlock = 128;
constexpr int kMaxR = 9, kMaxN = 3 * kMaxR + 3, kTerms = 64;
constexpr int kNF = kMaxN + 2;
// doubles of shared memory per warp: vertices (n+1) x 32, per-lane vertex
// costs, the evaluation point, band terms (residual^2, K, bottom share),
// per-region Rrs(490/550/640), final details and per-region bottom shares
constexpr int kSmem = (kMaxN + 1) * 32 + kNF * 32 + 32 + 3 * kTerms + 3 * 16 + 8 + 16;

// The 3 x 3 neighbourhood of pixel (i, j): region pixel indexes in the
// reference's order, their count and the origin's slot.
__device__ __forceinline__ int regions_of(const RegionArgs &a, int i, int j, int64_t (&rp)[kMaxR],
                                          int &origin) {
  const int nb = a.fp.n_bands;
  int R = 0;
  origin = 0;
  for (int ii = -1; ii <= 1; ii++) {
    const int iii = i + ii < 0 ? 0 : (i + ii > a.nrows - 1 ? a.nrows - 1 : i + ii);
    for (int jj = -1; jj <= 1; jj++) {
      const int jjj = j + jj < 0 ? 0 : (j + jj > a.ncols - 1 ? a.ncols - 1 : j + jj);
      const int64_t q = (int64_t)iii * a.ncols + jjj;
      bool nodata = false;
      for (int b = 0; b < nb; b++) {
        const float v = a.grid[q * nb + b];
        const float diff = __fsub_rn(v, a.fp.nodata);
        const double big = fabs((double)v) < fabs((double)a.fp.nodata) ? fabs((double)a.fp.nodata)
                                                                       : fabs((double)v);
        if (fabs((double)diff) <= big * (double)1.0e-6f) nodata = true;
      }
      if (i == iii && j == jjj) origin = R;
      if (!nodata) rp[R++] = q;
    }
  }
  return R;
}

__global__ void __launch_bounds__(kBlock) region_kernel(const __grid_constant__ RegionArgs a) {
  extern __shared__ double smem[];
  const FitParams &fp = a.fp;
  const SceneConsts &sc = a.sc;
  const photic_outputs &o = a.out;
  const int nb = fp.n_bands;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double *base = smem + warp * kSmem;
  double *V = base, *Fb = V + (kMaxN + 1) * 32, *X = Fb + kNF * 32, *dd = X + 32,
         *kk = dd + kTerms, *io = kk + kTerms, *s490 = io + kTerms, *s550 = s490 + 16,
         *s640 = s550 + 16, *misc = s640 + 16;

  NmGroup<0, 1, 32, 32> m;
  m.V = V;
  m.Fv = Fb + lane;
  m.X = X;
  m.gl = lane;
  m.gmask = kFull;
  m.clear();
  m.nrt = 6;

  const int64_t npix = (int64_t)a.nrows * a.ncols;
  const double early = fp.early_exit_per_scene * (double)(float)1;

  for (;;) {
    unsigned long long t = 0;
    if (lane == 0) t = atomicAdd(a.queue, 1ull);
    t = __shfl_sync(kFull, t, 0);
    if (t >= (unsigned long long)npix) break;
    const int64_t p = (int64_t)t;
    const int i = (int)(p / a.ncols), j = (int)(p % a.ncols);

    // the pixel loop's mask test on the centre (model/samodel.c:933-947)
    bool masked = false;
    for (int b = 0; b < nb; b++) {
      const float v = a.grid[p * nb + b];
      const float diff = __fsub_rn(v, fp.nodata);
      const double big = fabs((double)v) < fabs((double)fp.nodata) ? fabs((double)fp.nodata)
                                                                   : fabs((double)v);
      if (fabs((double)diff) <= big * (double)1.0e-6f || v < 0.0f) masked = true;
    }
    if (masked) {
      if (lane == 0) {
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
      }
      continue;
    }

    // ---- set-up: regions, per-term inputs, per-region shape values
    int64_t rp[kMaxR];
    int origin = 0;
    const int R = regions_of(a, i, j, rp, origin);
    const int N = 3 * R + 3, nterm = R * nb;
    m.nrt = N;
    double my_rrs[2] = {0.0, 0.0}, my_pw[2] = {0.0, 0.0};
    int my_r[2] = {0, 0}, my_b[2] = {0, 0};
    bool my_on[2] = {false, false};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int tau = lane + 32 * h;
      if (tau < nterm) {
        const int r = tau / nb, b = tau % nb;
        double r4[4];
#pragma unroll
        for (int c = 0; c < 4; c++) r4[c] = c < nb ? (double)a.grid[rp[r] * nb + c] : 0.0;
        double r440 = interp_plan<4>(fp.plan[0], r4);
        const double r490 = interp_plan<4>(fp.plan[1], r4);
        if (r440 < 0.0) r440 = 0.0001;
        const double chi = r440 / r490;
        double Y = 3.44 * (1.0 - 3.17 * fm::exp_t(-2.01 * chi));
        if (Y < 0.0) Y = 0.0;
        if (Y > 2.5) Y = 2.5;
        my_rrs[h] = r4[b];
        my_pw[h] = pow(sc.ratio440[b], Y);
        my_r[h] = r;
        my_b[h] = b;
        my_on[h] = true;
      }
    }
    if (lane < R) {
      double r4[4];
#pragma unroll
      for (int c = 0; c < 4; c++) r4[c] = c < nb ? (double)a.grid[rp[lane] * nb + c] : 0.0;
      s490[lane] = interp_plan<4>(fp.plan[1], r4);
      s550[lane] = interp_plan<4>(fp.plan[2], r4);
      s640[lane] = interp_plan<4>(fp.plan[3], r4);
    }
    __syncwarp();
    // mean measured Rrs over all region-bands, in the cost's order
    double tot = 0.0;
    if (lane == 0) {
      for (int r = 0; r < R; r++)
        for (int b = 0; b < nb; b++) tot = tot + (double)a.grid[rp[r] * nb + b];
    }
    tot = __shfl_sync(kFull, tot, 0);
    const double mean = tot / (double)nterm;

    // cold start of the lane's coordinate (model/samodel.c:2249-2353)
    auto cold = [&](double hs) {
      const int c = lane;
      double st = 0.0, sp = 0.0;
      if (c < R) {
        st = hs;
        sp = 1.25 * st;
      } else if (c < 2 * R) {
        double m490 = 0.0;
        for (int r = 0; r < R; r++) m490 += s490[r];
        m490 /= (double)R * 1;
        st = 100.0 * 4.0 * m490;
        sp = 1.5 * st;
      } else if (c < 3 * R) {
        st = 1.0;
        sp = 0.5 * st;
      } else if (c < N) {
        double m490 = 0.0, m550 = 0.0, m640 = 0.0;
        for (int r = 0; r < R; r++) {
          m490 += s490[r];
          m550 += s550[r];
          m640 += s640[r];
        }
        m490 /= (double)R;
        m550 /= (double)R;
        m640 /= (double)R;
        const double P = 100.0 * 0.072 * pow(m490 / m550, -1.7);
        st = c == 3 * R ? P : c == 3 * R + 1 ? 1.5 * P : 100.0 * 30.0 * fp.aw640 * m640;
        sp = 2.0 * st;
      }
      m.start[0] = st;
      m.step[0] = sp;
    };

    const double var_limit = fp.reqmin * (double)N;
    const int32_t guard_cap = (fp.n_hstarts + 1) * (fp.kcount + 8 * N + 16);
    int32_t kst = 0, total = 0, kept_evals = 0, kept_start = 0, kept_fault = 0, guard = 0;
    double lowest = 1.0e4, best = 0.0;
    bool final_eval = false, bad = false;
    cold(fp.hstarts[0]);
    m.begin(var_limit, fp.konvge, fp.kcount);

    for (;;) {
      __syncwarp();
      // ---- band terms at X
#pragma unroll
      for (int h = 0; h < 2; h++) {
        if (!my_on[h]) continue;
        const int r = my_r[h], b = my_b[h], tau = lane + 32 * h;
        const double H = fabs(X[r]);
        const double P = 0.01 * fabs(X[3 * R]);
        const double Gg = 0.01 * fabs(X[3 * R + 1]);
        const double Xx = 0.01 * fabs(X[3 * R + 2]);
        const double B = 0.01 * fabs(X[R + r]);
        double q = fabs(X[2 * R + r]), q_sum = 0.0;
        q_sum += q;
        q /= q_sum;
        const double rho = q * B * sc.refl[b];
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
        double M = sc.sec_sun + DuC * sc.sec_view;
        const double rrs_C = rrs_dp * (1.0 - fm::exp_t(-M * Kb * H));
        M = sc.sec_sun + DuB * sc.sec_view;
        const double rrs_B = fm::div_by(rho, kPi, fm::kInvPi) * fm::exp_t(-M * Kb * H);
        const double rrs = rrs_C + rrs_B;
        const double Rm = 0.5 * rrs / (1.0 - 1.5 * rrs);
        const double d = Rm - my_rrs[h];
        dd[tau] = d * d;
        kk[tau] = Kb;
        if (final_eval) io[tau] = rrs_B / rrs;
      }
      // each region's bottom share |100 B| |q| / q_sum on its own lane (the
      // division is the costly part of the bottom-continuity term)
      if (lane < R) {
        double qs = 0.0;
        qs += fabs(X[2 * R + lane]);
        misc[8 + lane] = fabs(X[R + lane]) * fabs(X[2 * R + lane]) / qs;
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
        // bottom continuity (one bottom type)
        th = dmean < 5.0 ? 0.25 : dmean < 10.0 ? 0.1 : dmean < 15.0 ? 0.05 : 0.01;
        double Eb = 0.0, bmean = 0.0, btotal = 0.0;
        nout = 0.0;
        for (int r = 0; r < R; r++) bmean += misc[8 + r];
        bmean /= (double)R;
        btotal += bmean;
        for (int r = 0; r < R; r++) {
          const double bt = misc[8 + r];
          if (bt < (1.0 - th) * bmean || bt > (1.0 + th) * bmean) {
            const double dv = bt - bmean;
            Eb += dv * dv;
            nout += 1.0;
          }
        }
        if (nout > 0.5) {
          bmean = btotal / ((double)1);
          Eb = 100.0 * sqrt(Eb / nout) / bmean;
        }
        // K terms: the origin's depth, the scene's K = the last region's
        double km = 1.0e4;
        for (int b = 0; b < nb; b++) {
          const double Kb = kk[(R - 1) * nb + b];
          if (__double2float_rn(Kb) != 0.0f && Kb < km) km = Kb;
        }
        double Ke = k_penalty_f64(fp.kp, fabs(X[origin]), km);
        if (km > 0.7) {
          const double dk = 4.0 * (km - 0.7);
          Ke = Ke + 100.0 * (dk * dk);
        }
        double model = 80.0 * E + 15.0 * Ed + 10.0 * Eb + 15.0 * Ke;
        model = fm::div_by(model, 120.0, fm::kInv120);
        y = model;
        if (final_eval) {
          double iod = 0.0, Kall = 1.0e4;
          for (int tau = 0; tau < nterm; tau++) iod = iod + io[tau];
          for (int b = 0; b < nb; b++) {
            const double Kb = kk[(R - 1) * nb + b];
            if (__double2float_rn(Kb) != 0.0f && Kb < Kall) Kall = Kb;
          }
          double q = fabs(X[3 * R - 1]), qs = 0.0;
          qs += q;
          q /= qs;
          misc[0] = E;
          misc[1] = model;
          misc[2] = q * (0.01 * fabs(X[2 * R - 1]));
          misc[3] = Kall == 1.0e4 ? 0.0 : Kall;
          misc[4] = 100.0 * iod / (double)nterm;
        }
      }
      y = __shfl_sync(kFull, y, 0);
      __syncwarp();

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
          if (o.depth) o.depth[p] = (float)depth;
          if (o.depth_f64) o.depth_f64[p] = depth;
          if (o.P) o.P[p] = (float)(0.01 * fabs(X[3 * R]));
          if (o.G) o.G[p] = (float)(0.01 * fabs(X[3 * R + 1]));
          if (o.X) o.X[p] = (float)(0.01 * fabs(X[3 * R + 2]));
          if (o.bottom_albedo) o.bottom_albedo[p] = (float)misc[2];
          if (o.model_error) o.model_error[p] = (float)misc[1];
          if (o.rrs_error) o.rrs_error[p] = (float)misc[0];
          if (o.K_min) o.K_min[p] = (float)misc[3];
          if (o.iod) o.iod[p] = (float)misc[4];
          if (o.evals) o.evals[p] = total;
          if (o.evals_kept) o.evals_kept[p] = kept_evals;
          if (o.status)
            o.status[p] = PHOTIC_PX_FITTED | (kept_fault == 0 ? PHOTIC_PX_CONVERGED : 0) |
                          (kept_start << 16) | (R << 24);
        }
        break;
      }
      if (++guard > guard_cap) {
        if (lane == 0) {
          atomicOr(a.error, PHOTIC_DEVERR_EVAL_CAP);
          if (o.status) o.status[p] = PHOTIC_PX_INVALID;
        }
        bad = true;
        break;
      }
      if (m.step_machine(y)) {
        // nelmin returned: keep the best start (model/samodel.c:2380-2405)
        const double ynewlo = m.F(m.lo);
        total += m.icount;
        bool finish = false;
        if (ynewlo < lowest) {
          lowest = ynewlo;
          best = m.xmin[0];
          kept_evals = m.icount;
          kept_start = kst;
          kept_fault = m.ifault;
          if (lowest < early) finish = true;  // model/samodel.c:2404
        }
        kst++;
        if (finish || kst >= fp.n_hstarts) {
          if (lane < N) X[lane] = best;  // re-evaluate at the kept optimum (:2413)
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
    (void)bad;
    __syncwarp();
  }
}

}  // namespace

size_t region_smem_bytes() { return (size_t)(kBlock / 32) * kSmem * sizeof(double); }

cudaError_t launch_region(const RegionArgs &a, int sms, int per_sm, cudaStream_t s) {
  const size_t bytes = region_smem_bytes();
  cudaError_t e =
      cudaFuncSetAttribute(region_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, region_kernel, kBlock, bytes);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  const int use = per_sm > 0 && per_sm < occ ? per_sm : occ;
  region_kernel<<<sms * use, kBlock, bytes, s>>>(a);
  return cudaGetLastError();
}

}  // namespace photic
