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
// chain mode, per warp: the measured bands 1..3 of every region and scene,
// the modelled Rrs of the final evaluation, the chain's P, G, X and state
constexpr int kChainD = 3 * kRS + kTerms + 3 * kMaxScenes + 24;
// the cost's staging, per warp: |H| and depth deviations per region, bottom
// deviations per (type, region), K penalty and smallest K per scene, mean
// share per type
constexpr int kStage = 64;

// Launch shapes: C coordinates per lane, vertex row stride CG.
template <int C, int CG>
struct Shape {
  static constexpr int kMaxN = C == 1 ? 32 : CG;
  static constexpr int kNF = kMaxN + 2;
  // doubles of shared memory per warp: vertices (n+1) x CG, the vertex
  // costs (one copy for the warp), the evaluation point, band terms (residual^2, K, bottom share of
  // the reflectance), per-region Rrs(490/550/640), final details and
  // per-(region, bottom) shares of the bottom-continuity term, and the
  // chain mode's arrays
  static constexpr int kSmem =
      (kMaxN + 1) * CG + kNF + 32 * C + 3 * kTerms + 3 * kRS + 8 + kShares + kChainD + kStage;
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

// ---- chain mode: samodel()'s loop with its lookup table (model/samodel.c:
// 649-1352) over the region fit.  A warp runs one chain (a contiguous slice
// of the sorted shallow pixels) as one thread of the reference runs its
// pixels: the table scan by the 32 lanes, a served pixel's outputs copied
// from its entry's pixel, a fit hot-started from the previous pixel when the
// last two were continuous, the entry and the adaptive thresholds.
//
// The chain's state, in the warp's shared memory, written by lane 0:
enum : int { G_DEPTH, G_KMIN, G_DPREV, G_KPREV, G_HEMP, G_MATCH, G_ENTRY, G_NMOD, G_NSKIP,
             G_TOTME, G_ERRTOT, G_ERRCNT, G_NOPT, G_TOTLUT, G_NCOMP, G_NPREV, G_HOT, G_K,
             G_KBEG, G_KEND, G_CHAIN, G_COUNT };
static_assert(G_COUNT <= 24, "chain state");
constexpr double kEps = (double)1.0e-4f;  // the reference's float epsilon (model/common.c:93)
constexpr double kContinuity = 0.1;       // :981
constexpr double kMinThreshold = 1.5;     // :892
constexpr double kMaxSkip = 0.9925;       // :880

// A new chain c (:871-899): empty table, thresholds MAX(1.5, 1.125 S), no
// previous pixel; h_empirical, which the reference leaves unset until a
// pixel with an empirical depth, is 0 (every bottom type fitted).
__device__ __forceinline__ void chain_begin(const RegionArgs &a, double *cst, double *cprev,
                                            int64_t c, int S) {
  for (int k = 0; k < G_COUNT; k++) cst[k] = 0.0;
  const double m0 = 1.125 * (double)S;
  cst[G_MATCH] = m0 > kMinThreshold ? m0 : kMinThreshold;
  cst[G_ENTRY] = cst[G_MATCH];
  cst[G_CHAIN] = (double)c;
  cst[G_KBEG] = (double)(c * a.n_shallow / a.n_chains);
  cst[G_KEND] = (double)((c + 1) * a.n_shallow / a.n_chains);
  cst[G_K] = cst[G_KBEG];
  for (int i = 0; i < 3 * kMaxScenes; i++) cprev[i] = 0.0;
}

// After a pixel, served or fitted (:1102-1211, the statistics restarting at
// every update, :1326-1352): the hot-start decision, the previous pixel,
// the thresholds every 0.1 % of the chain.  Lane 0.
__device__ __forceinline__ void chain_post(const RegionArgs &a, double *cst, double me) {
  const double depth = cst[G_DEPTH], kmin = cst[G_KMIN];
  const double dprev = cst[G_DPREV], kprev = cst[G_KPREV];
  cst[G_HOT] = (fabs(depth - dprev) / (kEps + dprev) < kContinuity &&
                fabs(kmin - kprev) / (kEps + kprev) < kContinuity)
                   ? 1.0
                   : 0.0;
  cst[G_DPREV] = depth;
  cst[G_KPREV] = kmin;
  cst[G_TOTME] = cst[G_TOTME] + me;
  cst[G_NMOD] = cst[G_NMOD] + 1.0;
  cst[G_NCOMP] += 1.0;
  const int nperc = (int)((1000.0 * cst[G_NCOMP]) / (cst[G_KEND] - cst[G_KBEG]));
  if ((double)nperc > cst[G_NPREV]) {
    double match = cst[G_MATCH], entry = cst[G_ENTRY];
    const double n_mod = cst[G_NMOD];
    if (cst[G_NOPT] > 0.0) {
      const double cnt = cst[G_ERRCNT];
      // vec_mean2_double (model/common.c:877-891) returns a float
      const double error_mean = (double)(float)(cnt > 0.0 ? cst[G_ERRTOT] / cnt : 0.0);
      match = match + (0.75 * error_mean + (0.25 * cst[G_TOTME]) / n_mod);
      match = match / 2.0;
      entry = match;
    }
    if (cst[G_NSKIP] / n_mod > kMaxSkip) {
      match = match * 0.75;
      entry = entry * 0.75;
    }
    cst[G_MATCH] = kMinThreshold > match ? kMinThreshold : match;
    cst[G_ENTRY] = kMinThreshold > entry ? kMinThreshold : entry;
    cst[G_NPREV] = (double)nperc;
    cst[G_TOTME] = 0.0;
    cst[G_NMOD] = 0.0;
    cst[G_NSKIP] = 0.0;
    cst[G_NOPT] = 0.0;
    cst[G_ERRTOT] = 0.0;
    cst[G_ERRCNT] = 0.0;
  }
  cst[G_K] += 1.0;
  if (a.chain_stats) {
    const int64_t c = (int64_t)cst[G_CHAIN];
    a.chain_stats[c * 4 + 2] = cst[G_MATCH];
    a.chain_stats[c * 4 + 3] = cst[G_ENTRY];
  }
}

// model_spectral_diff_mean (model/samodel.c:2792-2842): bands 1..3 below
// n_bands, the measured (meas, scene-major) and the entry's modelled Rrs
// (rm, region-major) averaged over the scenes and regions where both are
// non-zero; the square by a multiply where the reference calls pow(x, 2).
__device__ __forceinline__ float glut_diff(const double *meas, const double *rm, int R, int S,
                                           int nb) {
  double error = 0.0;
  int n_total = 0;
  for (int k = 1; k <= 3; k++) {
    if (k >= nb) break;
    double current = 0.0, previous = 0.0, nobs = 0.0;
    for (int s = 0; s < S; s++)
      for (int r = 0; r < R; r++) {
        const double mv = meas[(s * R + r) * 3 + k - 1], lv = rm[(r * S + s) * 3 + k - 1];
        if ((float)mv != 0.0f && (float)lv != 0.0f) {
          current = current + mv;
          previous = previous + lv;
          nobs = nobs + 1.0;
        }
      }
    if (nobs > 0.5) {
      current = current / nobs;
      previous = previous / nobs;
    }
    const double t = (current - previous) / current;
    error = error + t * t;
    n_total++;
  }
  error = 100.0 * sqrt(error / (double)n_total);
  return (float)error;
}

// A served pixel's outputs (partial_copy_md, model/samodel.c:3031-3139, then
// the grids of :1118-1166): those of the pixel whose fit the entry holds,
// with the spectral difference as model error; the lanes copy one field
// each.
__device__ __noinline__ void serve_copy(const RegionArgs &a, int64_t p, int64_t src, float diff,
                                        int S, int lane) {
  const photic_outputs &o = a.out;
  for (int f = lane; f < 15 + 3 * S; f += 32) {
    if (f == 0) { if (o.depth) o.depth[p] = o.depth[src]; }
    else if (f == 1) { if (o.depth_f64) o.depth_f64[p] = o.depth_f64[src]; }
    else if (f == 2) { if (o.bottom_albedo) o.bottom_albedo[p] = o.bottom_albedo[src]; }
    else if (f == 3) { if (o.model_error) o.model_error[p] = diff; }
    else if (f == 4) { if (o.rrs_error) o.rrs_error[p] = o.rrs_error[src]; }
    else if (f == 5) { if (o.K_min) o.K_min[p] = o.K_min[src]; }
    else if (f == 6) { if (o.iod) o.iod[p] = o.iod[src]; }
    else if (f == 7) { if (o.evals) o.evals[p] = 0; }
    else if (f == 8) { if (o.evals_kept) o.evals_kept[p] = 0; }
    else if (f == 9) {
      if (o.status)
        o.status[p] = PHOTIC_PX_FITTED | PHOTIC_PX_SERVED |
                      (o.status[src] & (PHOTIC_PX_CONVERGED | (0xF << 24)));
    } else if (f == 10) { if (a.source) a.source[p] = src; }
    else if (f == 11) { if (o.bottom_type) o.bottom_type[p] = o.bottom_type[src]; }
    else if (f < 15) {
      if (o.bottom_percent) o.bottom_percent[p * 3 + f - 12] = o.bottom_percent[src * 3 + f - 12];
    } else {
      const int j = f - 15, s = j % S;
      float *v = j < S ? o.P : (j < 2 * S ? o.G : o.X);
      if (v) v[p * S + s] = v[src * S + s];
    }
  }
}

// (One block per SM as the launch bound's minimum: without it the compiler
// held the kernel to 128 registers and spilled.)
template <int C, int CG, int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1) region_kernel(const __grid_constant__ RegionArgs a) {
  using Sh = Shape<C, CG>;
  constexpr int kMaxN = Sh::kMaxN, kNF = Sh::kNF;
  extern __shared__ double smem[];
  const FitParams &fp = a.fp;
  const SceneConsts &sc = a.sc;
  const photic_outputs &o = a.out;
  const int nb = fp.n_bands, S = a.n_scenes;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double *base = smem + warp * Sh::kSmem;
  double *V = base, *Fb = V + (kMaxN + 1) * CG, *X = Fb + kNF, *dd = X + 32 * C,
         *kk = dd + kTerms, *io = kk + kTerms, *s490 = io + kTerms, *s550 = s490 + kRS,
         *s640 = s550 + kRS, *misc = s640 + kRS;
  double *share = misc + 8;
  double *meas = share + kShares, *rmv = meas + 3 * kRS, *cprev = rmv + kTerms,
         *cst = cprev + 3 * kMaxScenes, *stg = cst + 24;
  const bool list = a.list_R != nullptr;
  // spectrum of scene s of region slot q (a pixel index of the grid, or a
  // region row of the list)
  auto spec = [&](int64_t q, int s) -> const float * {
    return list ? a.list_rrs + (q * S + s) * nb : a.grid + ((int64_t)s * a.npix + q) * nb;
  };

  NmGroup<0, C, 32, CG, true> m;
  m.V = V;
  m.Fv = Fb;
  m.X = X;
  m.gl = lane;
  m.gmask = kFull;
  m.clear();
  m.nrt = 6;

  const double early = fp.early_exit_per_scene * (double)(float)S;
  const double kNaN = __longlong_as_double(0x7ff8000000000000LL);
  const bool chained = a.order != nullptr;
  if (chained) {
    if (lane == 0) {
      cst[G_K] = 0.0;
      cst[G_KEND] = 0.0;
    }
    __syncwarp();
  }

  for (;;) {
    int64_t p = 0;
    int64_t rp[kMaxR];
    int origin = 0, R = 0;
    bool hot = false;
    // the depth start (NaN: the cold starts) and the depth that picks sand
    // alone above 8 m (model/samodel.c:1781, 1826-1830)
    double hemp = kNaN, hbot = kNaN;
    if (chained) {
      // ---- the chain's next pixel that its table cannot serve
      bool done = false;
      for (;;) {
        if (cst[G_K] >= cst[G_KEND]) {
          unsigned long long c = 0;
          if (lane == 0) c = atomicAdd(a.queue, 1ull);
          c = __shfl_sync(kFull, c, 0);
          if (c >= (unsigned long long)a.n_chains) {
            done = true;
            break;
          }
          __syncwarp();
          if (lane == 0) chain_begin(a, cst, cprev, (int64_t)c, S);
          __syncwarp();
          continue;
        }
        p = a.order[(int64_t)cst[G_K]];
        R = regions_of(a, p, rp, origin);
        // the pixel's empirical depth (:955-976)
        bool emp_present = false;
        double h_emp = 0.0;
        if (a.emp) {
          const float e = a.emp[p];
          if (!nodata_value(e, a.emp_nodata)) {
            emp_present = true;
            h_emp = (double)e > -1.0 ? 1.0 : fabs((double)e);
          }
        }
        // measured bands 1..3 of every region and scene, scene-major
        for (int t = lane; t < R * S * 3; t += 32) {
          const int s = t / (R * 3), r = (t / 3) % R, k = t % 3 + 1;
          meas[t] = k < nb ? (double)spec(rp[r], s)[k] : 0.0;
        }
        __syncwarp();
        if (lane == 0 && a.emp) {
          if (emp_present) cst[G_HEMP] = h_emp;
          else cst[G_HOT] = 0.0;
        }
        // lookup (:980-999): among the entries with the pixel's region
        // count and within 10 % of the previous pixel's depth and K_min,
        // the first slot of least spectral difference
        const int64_t c = (int64_t)cst[G_CHAIN];
        const int64_t tl = (int64_t)cst[G_TOTLUT];
        const int64_t n_in = tl < a.cap ? tl : a.cap;
        const double dep = cst[G_DEPTH], km = cst[G_KMIN];
        const double *ring = a.ring + (size_t)c * a.cap * a.entry_stride;
        double bestd = 1.0e4;
        int64_t pos = 0;
        for (int64_t j = lane; j < n_in; j += 32) {
          const double *e = ring + j * a.entry_stride;
          if ((int)e[0] == R && fabs(e[1] - dep) / (dep + kEps) < kContinuity &&
              fabs(e[2] - km) / (km + kEps) < kContinuity) {
            const double d = (double)glut_diff(meas, e + 3 + 3 * S, R, S, nb);
            if (d < bestd) {
              bestd = d;
              pos = j;
            }
          }
        }
#pragma unroll
        for (int w = 16; w > 0; w >>= 1) {
          const double ob = __shfl_xor_sync(kFull, bestd, w);
          const int64_t op = __shfl_xor_sync(kFull, pos, w);
          if (ob < bestd || (ob == bestd && op < pos)) {
            bestd = ob;
            pos = op;
          }
        }
        __syncwarp();
        if (bestd > cst[G_MATCH] || n_in == 0) {
          // a fit (:1008-1063), hot when the last two pixels were
          // continuous (:2234-2241: the empirical depth keeps its start)
          hot = cst[G_HOT] != 0.0;
          hbot = cst[G_HEMP];
          hemp = emp_present ? h_emp : (hot ? cst[G_DPREV] : kNaN);
          break;
        }
        // served (:1066-1073): the entry's pixel's outputs
        const int64_t src = a.ring_src[(size_t)c * a.cap + pos];
        const double *e = ring + pos * a.entry_stride;
        serve_copy(a, p, src, (float)bestd, S, lane);
        for (int i = lane; i < 3 * S; i += 32) cprev[i] = e[3 + i];
        __syncwarp();
        if (lane == 0) {
          cst[G_DPREV] = cst[G_DEPTH];
          cst[G_KPREV] = cst[G_KMIN];
          cst[G_DEPTH] = e[1];
          cst[G_KMIN] = e[2];
          cst[G_NSKIP] = cst[G_NSKIP] + 1.0;
          if (a.chain_stats) a.chain_stats[c * 4 + 0] += 1.0;
          chain_post(a, cst, bestd);
        }
        __syncwarp();
      }
      if (done) break;
    } else {
      unsigned long long t = 0;
      if (lane == 0) t = atomicAdd(a.queue, 1ull);
      t = __shfl_sync(kFull, t, 0);
      if (t >= (unsigned long long)a.npix) break;
      p = (int64_t)t;

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
      R = regions_of(a, p, rp, origin);
      if (a.h_emp) hemp = hbot = a.h_emp[p];
    }

    // ---- set-up: bottom types, per-term inputs
    int nbt = a.n_bottoms;
    if (!isnan(hbot) && hbot > 8.0) nbt = 1;  // model/samodel.c:1781, 1826-1830
    const int N = R + 2 * nbt * R + 3 * S, nterm = R * S * nb;
    const int qo = R + R * nbt, off = R + 2 * nbt * R;
    if (R < 1 && a.list_R) {
      // a problem without regions (md->n_regions == 0: the reference's
      // loops skip it, model/samodel.c:951-953, 1428-1430)
      if (lane == 0) write_masked(o, p, S, PHOTIC_PX_MASKED);
      __syncwarp();
      continue;
    }
    if (R < 1 || N > kMaxN || nterm > kTerms || R * S > kRS) {
      if (lane == 0) {
        atomicOr(a.error, PHOTIC_DEVERR_EVAL_CAP);
        write_masked(o, p, S, PHOTIC_PX_INVALID);
        if (chained) cst[G_K] += 1.0;
      }
      __syncwarp();
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
        if (hot && c >= off && c < N) {  // the previous fit's P, G, X (:2288-2309)
          st = cprev[c - off];
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
    bool final_eval = eval_only, fitted = false;
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
          if (chained) rmv[tau] = Rm;
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
      // ---- the cost (model/samodel.c:2432-2759).  Every sum keeps the
      // reference's order on one lane; the sums that do not depend on one
      // another run on different lanes together, and the terms they add
      // (|H| per region, the squared deviations, each scene's K penalty)
      // are formed by the lanes in parallel.  An outside-the-band term that
      // the reference skips is added here as +0, which leaves every partial
      // sum unchanged (the terms are >= 0).
      double *habs = stg, *dv2d = stg + 9, *dv2b = stg + 18, *kpen = stg + 45, *bmv = stg + 53,
             *kms = stg + 56;
      if (lane < R) habs[lane] = fabs(X[lane]);
      if (lane < S) {  // each scene's smallest K over the last region's bands (:2696-2701)
        double km = 1.0e4;
        for (int b = 0; b < nb; b++) {
          const double Kb = kk[((R - 1) * S + lane) * nb + b];
          if (__double2float_rn(Kb) != 0.0f && Kb < km) km = Kb;
        }
        kms[lane] = km;
      }
      __syncwarp();
      // ordered sums: lane 0 the squared residuals (:2571), lane 1 the
      // depths (:2597-2600), lane 2 + k the bottom shares of type k (:2652)
      double z = 0.0;
      {
        const double *src = dd;
        int cnt = 0, str = 1;
        if (lane == 0) {
          cnt = nterm;
        } else if (lane == 1) {
          src = habs;
          cnt = R;
        } else if (lane < 2 + nbt) {
          src = share + (lane - 2);
          cnt = R;
          str = nbt;
        }
        for (int i = 0; i < cnt; i++) z = z + src[i * str];
      }
      const double err = __shfl_sync(kFull, z, 0);
      const double dmean = __shfl_sync(kFull, z, 1) / (double)R;
      if (lane >= 2 && lane < 2 + nbt) bmv[lane - 2] = z / (double)R;
      const double thd = dmean < 4.0 ? 0.4 : dmean < 8.0 ? 0.2 : dmean < 12.0 ? 0.1 : 0.05;
      const double thb = dmean < 5.0 ? 0.25 : dmean < 10.0 ? 0.1 : dmean < 15.0 ? 0.05 : 0.01;
      bool outd = false, outb = false;
      if (lane < R) {  // depth continuity, one region per lane (:2604-2617)
        const double h = habs[lane];
        outd = h < (1.0 - thd) * dmean || h > (1.0 + thd) * dmean;
        const double dv = h - dmean;
        dv2d[lane] = outd ? dv * dv : 0.0;
      }
      __syncwarp();
      if (lane < nbt * R) {  // bottom continuity, one (type, region) per lane (:2655-2668)
        const int k = lane / R, r = lane % R;
        const double bm = bmv[k], bt = share[r * nbt + k];
        outb = bt < (1.0 - thb) * bm || bt > (1.0 + thb) * bm;
        const double dv = bt - bm;
        dv2b[lane] = outb ? dv * dv : 0.0;
      }
      if (lane < S) kpen[lane] = k_penalty_f64(fp.kp, habs[origin], kms[lane]);
      const double nd = (double)__popc(__ballot_sync(kFull, outd));
      const double nbo = (double)__popc(__ballot_sync(kFull, outb));
      __syncwarp();
      // ordered sums: lane 0 the depth deviations, lane 1 the bottom
      // deviations (type-major), lane 2 the scenes' K penalties, lane 3 the
      // types' mean shares
      double z2 = 0.0;
      {
        const double *src = dv2d;
        int cnt = 0;
        if (lane == 0) {
          cnt = R;
        } else if (lane == 1) {
          src = dv2b;
          cnt = nbt * R;
        } else if (lane == 2) {
          src = kpen;
          cnt = S;
        } else if (lane == 3) {
          src = bmv;
          cnt = nbt;
        }
        for (int i = 0; i < cnt; i++) z2 = z2 + src[i];
      }
      double Ed = __shfl_sync(kFull, z2, 0), Eb = __shfl_sync(kFull, z2, 1);
      double Ke = __shfl_sync(kFull, z2, 2);
      const double btotal = __shfl_sync(kFull, z2, 3);
      double y = 0.0;
      if (lane == 0) {
        const double E = 100.0 * sqrt(fm::div_count(err, nterm)) / mean;
        if (nd > 0.5) Ed = 100.0 * sqrt(Ed / nd) / dmean;
        if (nbo > 0.5) {
          const double bmean = btotal / ((double)nbt);
          Eb = 100.0 * sqrt(Eb / nbo) / bmean;
        }
        // the very-high-K term on the last scene's K (:2728-2732)
        const double km = kms[S - 1];
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
          misc[6] = depth;
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
                          (hot ? PHOTIC_PX_HOT : 0) | (kept_start << 16) | (R << 24);
        }
        if (a.list_params)
          for (int c = lane; c < N; c += 32) a.list_params[p * a.eval_stride + c] = X[c];
        fitted = true;
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
    if (chained) {
      // the fit's P, G, X for the next hot start (:2086-2099); the entry
      // (:1035-1063): region count, depth, K_min, P, G, X and the modelled
      // Rrs of bands 1..3 when the model error is below the entry
      // threshold and the depth below 32 m, into the oldest slot
      const int64_t c = (int64_t)cst[G_CHAIN];
      const double depth = misc[6], kmin = misc[3], me = misc[1];
      const bool ins = fitted && me < cst[G_ENTRY] && depth < 32.0;
      const int64_t slot = (int64_t)cst[G_TOTLUT] % a.cap;
      if (fitted)
        for (int i = lane; i < 3 * S; i += 32) cprev[i] = fabs(X[off + i]);
      __syncwarp();
      if (ins) {
        double *e = a.ring + ((size_t)c * a.cap + slot) * a.entry_stride;
        for (int i = lane; i < 3 * S; i += 32) e[3 + i] = cprev[i];
        for (int t = lane; t < R * S * 3; t += 32) {
          const int r = t / (S * 3), s = (t / 3) % S, k = t % 3 + 1;
          e[3 + 3 * S + t] = k < nb ? rmv[(r * S + s) * nb + k] : 0.0;
        }
        if (lane == 0) {
          e[0] = (double)R;
          e[1] = depth;
          e[2] = kmin;
          a.ring_src[(size_t)c * a.cap + slot] = p;
        }
      }
      __syncwarp();
      if (lane == 0) {
        if (fitted) {
          if (a.source) a.source[p] = -1;
          cst[G_DEPTH] = depth;
          cst[G_KMIN] = kmin;
          cst[G_NOPT] += 1.0;
          if ((float)me != 0.0f) {  // vec_mean2_double leaves zeros out
            cst[G_ERRTOT] = cst[G_ERRTOT] + me;
            cst[G_ERRCNT] += 1.0;
          }
          if (ins) cst[G_TOTLUT] += 1.0;
          if (a.chain_stats) a.chain_stats[c * 4 + 1] += 1.0;
          chain_post(a, cst, me);
        } else {
          cst[G_K] += 1.0;  // an invalid pixel leaves the chain's state alone
        }
      }
      __syncwarp();
    }
  }
}

// warps: when non-NULL, only the number of resident warps is returned.
template <int C, int CG, int BLOCK>
cudaError_t launch_shape(const RegionArgs &a, int sms, int per_sm, cudaStream_t s,
                         int64_t *warps) {
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
  if (warps) {
    *warps = grid * (BLOCK / 32);
    return cudaSuccess;
  }
  const int64_t units = a.order ? a.n_chains : a.npix;  // chains, or pixels
  const int64_t need = (units + BLOCK / 32 - 1) / (BLOCK / 32);
  if (grid > need) grid = need;
  k<<<(int)grid, BLOCK, bytes, s>>>(a);
  return cudaGetLastError();
}

// One thread per sample: the sampled pixel's regions in extract_Rrs_data's
// order with the perturbation of the depth-uncertainty refit (:1426-1427,
// 3003-3006: value + n R_sigma when n is not within 1e-6 of 0, in double,
// stored as float); no pixel: no regions.
__global__ void region_samples_kernel(const __grid_constant__ RegionSampleArgs a) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= a.ns) return;
  const int64_t p = a.sample_pixel[g];
  const int S = a.n_scenes, nb = a.n_bands;
  if (p < 0) {
    a.list_R[g] = 0;
    a.list_origin[g] = 0;
    return;
  }
  const int64_t npix = (int64_t)a.nrows * a.ncols;
  const int i = (int)(p / a.ncols), j = (int)(p % a.ncols), w = a.n_spatial - 1;
  const float n = a.sample_n[g];
  const bool move = !(fabsf(n - 0.0f) <= fabsf(n) * 1.0e-6f);
  int R = 0, origin = 0;
  for (int ii = -w; ii <= w; ii++) {
    const int iii = i + ii < 0 ? 0 : (i + ii > a.nrows - 1 ? a.nrows - 1 : i + ii);
    for (int jj = -w; jj <= w; jj++) {
      const int jjj = j + jj < 0 ? 0 : (j + jj > a.ncols - 1 ? a.ncols - 1 : j + jj);
      const int64_t q = (int64_t)iii * a.ncols + jjj;
      bool nodata = false;
      for (int s = 0; s < S && !nodata; s++)
        for (int b = 0; b < nb; b++) {
          const float refl = a.grid[(s * npix + q) * nb + b];
          if (nodata_value(refl, a.nodata)) {
            nodata = true;
            break;
          }
          double v = (double)refl;
          if (move) v += (double)n * a.r_sigma[s * 8 + b];
          a.list_rrs[((g * kMaxR + R) * S + s) * nb + b] = (float)v;
        }
      if (i == iii && j == jjj) origin = R;
      if (!nodata) R++;
    }
  }
  a.list_R[g] = R;
  a.list_origin[g] = origin;
}

}  // namespace

cudaError_t launch_region_samples(const RegionSampleArgs &a, cudaStream_t s) {
  if (a.ns <= 0) return cudaSuccess;
  region_samples_kernel<<<(unsigned)((a.ns + 127) / 128), 128, 0, s>>>(a);
  return cudaGetLastError();
}

int region_max_params(int max_regions, int n_bottoms, int n_scenes) {
  return max_regions + 2 * n_bottoms * max_regions + 3 * n_scenes;
}

cudaError_t launch_region(const RegionArgs &a, int max_params, int sms, int per_sm,
                          cudaStream_t s, int64_t *warps) {
  if (max_params <= Shape<1, 32>::kMaxN) return launch_shape<1, 32, 128>(a, sms, per_sm, s, warps);
  if (max_params <= Shape<3, kRegionMaxParams>::kMaxN)
    return launch_shape<3, kRegionMaxParams, 32>(a, sms, per_sm, s, warps);
  if (max_params <= Shape<3, 96>::kMaxN) return launch_shape<3, 96, 32>(a, sms, per_sm, s, warps);
  return cudaErrorInvalidValue;
}

}  // namespace photic
