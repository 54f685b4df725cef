// photic_lut.cu -- samodel()'s pixel loop with its dynamic lookup table
// (LUT 1, model/samodel.c:649-660, 701-773, 901-1215), one scene, one
// region, one bottom type.
//
// Order.  The shallow pixels (no band nodata or negative, :933-947) are
// sorted ascending by the spectral index |(Rrs_1, Rrs_2, Rrs_3)| (the blue,
// green and red bands, :711-745), times the spectral angle to the scene's
// noise spectrum when every band's noise is at least 1e-6 (:749-767).  The
// index is a float, sorted over every pixel by glibc's merge-sort qsort
// (:772, model/common.c:180-209): ties keep pixel order, so a stable radix
// sort of the shallow pixels gives the same order -- except where a key is
// NaN (a pixel whose blue, green and red are all nodata or zero, under the
// spectral angle), which the comparator calls equal to everything; then the
// reference's own merge tree is replayed level by level.
//
// Chains.  The sorted list is cut into contiguous slices.  Each slice runs
// the reference's loop exactly as one of its OpenMP threads runs the pixels
// it is given -- its own table of at most n_lut entries, its own previous
// pixel for the continuity tests and the hot start, its own adaptive
// thresholds updated every 0.1 % of the slice -- so one slice is the
// reference on one thread, and tens of thousands of slices are the same
// loop with the GPU's lanes as threads.
//
// Kernel.  Persistent, one lane per chain at a time (chains come from an
// atomic queue).  A lane whose chain needs its next pixel hands the warp
// the lookup: the 32 lanes scan the chain's table slots j = lane,
// lane + 32, ... (continuity tests, then model_spectral_diff_mean,
// :2792-2842) and reduce to the first slot of least difference.  A served
// pixel copies the entry's outputs (partial_copy_md, :3031-3139) and the
// warp moves on to the chain's next pixel; a pixel the table cannot serve
// starts a Nelder-Mead fit on its lane -- hot-started from the previous
// pixel when the last two pixels were continuous (:2234-2309) -- and the
// lanes evaluate their fits' costs together as the batched inversion does
// (photic_invert.cu).  When a fit ends, its lane enters it into the oldest
// slot if its model error is below the entry threshold and its depth below
// 32 m (:1035-1063) and carries on with its chain.
//
// Arithmetic: FP64 in the reference's order (--fmad=false); the spectral
// difference squares with a multiply where the reference calls pow(x, 2)
// (glibc's pow differs from the correctly rounded square in the last bit
// for about 1 in 1200 arguments, and the difference is then rounded to
// float).
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_kernels.h"
#include "photic_prec64.cuh"

namespace photic {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kN = kPrecN;
using P = PrecF64;
constexpr int kLutBlock = 256;
// the reference's float global epsilon (model/common.c:93), as a double
constexpr double kEps = (double)1.0e-4f;
constexpr double kContinuity = 0.1;     // :981
constexpr double kMinThreshold = 1.5;   // min_lut_match_threshold (:892)
constexpr double kMaxSkip = 0.9925;     // max_preferable_skip (:880)

// approx_equal (model/common.c:392-394): float arguments, double product
__device__ __forceinline__ bool ref_approx_eq(float a, float b, float eps) {
  const float d = __fsub_rn(a, b);
  const double fa = fabs((double)a), fb = fabs((double)b);
  return fabs((double)d) <= (fa < fb ? fb : fa) * (double)eps;
}

// ---------------------------------------------------------------------------
// Order
// ---------------------------------------------------------------------------
// The masked outputs of the general loop: the region fit's layout, with P,
// G, X per scene and the bottom shares.
__device__ void write_masked_general(const photic_outputs &o, int64_t p, int S) {
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
  if (o.status) o.status[p] = PHOTIC_PX_MASKED;
  if (o.bottom_percent)
    for (int k = 0; k < 3; k++) o.bottom_percent[p * 3 + k] = 0.0f;
  if (o.bottom_type) o.bottom_type[p] = 0.0f;
}

__global__ void lut_key_kernel(LutKeyArgs a) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npix) return;
  const int S = a.n_scenes;
  bool masked = false;
  for (int s = 0; s < S; s++) {  // every band of every scene (:933-947)
    const float *r = a.rrs + (s * a.npix + p) * a.n_bands;
    for (int b = 0; b < a.n_bands; b++)
      if (band_masked(r[b], a.nodata)) masked = true;
  }
  a.flags[p] = masked ? 0 : 1;
  a.idx[p] = p;
  if (masked) {
    if (a.general) write_masked_general(a.out, p, S);
    else write_masked(a.out, p);
    if (a.source) a.source[p] = -2;
  }
  if (a.emp) {  // the empirical depth itself (:708-710)
    a.keys[p] = a.emp[p];
    return;
  }
  // :711-745 -- float sums over the scenes, squares and root in double,
  // stored as float
  float bs = 0.0f, gs = 0.0f, rs = 0.0f;
  for (int s = 0; s < S; s++) {
    const float *r = a.rrs + (s * a.npix + p) * a.n_bands;
    if (a.n_bands > 1 && !ref_approx_eq(r[1], a.nodata, 1.0e-6f)) bs = __fadd_rn(bs, r[1]);
    if (a.n_bands > 2 && !ref_approx_eq(r[2], a.nodata, 1.0e-6f)) gs = __fadd_rn(gs, r[2]);
    if (a.n_bands > 3 && !ref_approx_eq(r[3], a.nodata, 1.0e-6f)) rs = __fadd_rn(rs, r[3]);
  }
  const double b2 = __dmul_rn((double)bs, (double)bs), g2 = __dmul_rn((double)gs, (double)gs),
               r2 = __dmul_rn((double)rs, (double)rs);
  float key = (float)sqrt(__dadd_rn(__dadd_rn(b2, g2), r2));
  if (a.use_noise) {  // :749-767
    const double bn = a.noise[0], gn = a.noise[1], rn = a.noise[2];
    double ang = __dadd_rn(__dadd_rn(__dmul_rn((double)bs, bn), __dmul_rn((double)gs, gn)),
                           __dmul_rn((double)rs, rn));
    const double nn = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(bn, bn), __dmul_rn(gn, gn)),
                                     __dmul_rn(rn, rn)));
    ang = ang / __dmul_rn((double)key, nn);
    ang = acos(ang);
    key = (float)__dmul_rn((double)key, ang);
  }
  a.keys[p] = key;
}

__global__ void gather_keys_kernel(const float *keys, const int64_t *idx, int64_t n,
                                   float *out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = keys[idx[k]];
}

__global__ void nan_count_kernel(const float *keys, int64_t n, unsigned long long *count) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n && isnan(keys[k])) atomicAdd(count, 1ull);
}

// One level of the reference's qsort (glibc's top-down merge sort: halves
// of n / 2 and n - n / 2, the merge taking the left element unless it
// compares greater), for key sets holding NaN: the comparator of
// sort_indexes_2d calls a NaN equal to everything, so the order depends on
// the merge tree and only the same tree reproduces it.  Thread t of level d
// owns the node reached from the root by the bits of t (most significant
// first: 0 left, 1 right) and merges its two halves from (kin, iin) into
// (kout, iout); nodes of fewer than two elements are copied.
__global__ void msort_level_kernel(const float *kin, const int64_t *iin, float *kout,
                                   int64_t *iout, int64_t n, int depth) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ((int64_t)1 << depth)) return;
  int64_t lo = 0, hi = n;
  for (int b = depth - 1; b >= 0; b--) {
    const int64_t mid = lo + (hi - lo) / 2;
    if ((t >> b) & 1) lo = mid;
    else hi = mid;
  }
  if (hi - lo < 2) {
    for (int64_t k = lo; k < hi; k++) {
      kout[k] = kin[k];
      iout[k] = iin[k];
    }
    return;
  }
  const int64_t mid = lo + (hi - lo) / 2;
  int64_t i = lo, j = mid, o = lo;
  while (i < mid && j < hi) {
    const float a = kin[i], b = kin[j];
    if (!(a > b)) {
      kout[o] = a;
      iout[o++] = iin[i++];
    } else {
      kout[o] = b;
      iout[o++] = iin[j++];
    }
  }
  while (i < mid) {
    kout[o] = kin[i];
    iout[o++] = iin[i++];
  }
  while (j < hi) {
    kout[o] = kin[j];
    iout[o++] = iin[j++];
  }
}

__global__ void gather_flags_kernel(const uint8_t *flags, const int64_t *idx, int64_t n,
                                    uint8_t *out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = flags[idx[k]];
}

// ---------------------------------------------------------------------------
// The pixel loop
// ---------------------------------------------------------------------------
// Per-lane chain state in shared memory, [field][lane] so that a warp's
// accesses to one field are conflict-free and any lane can read the state
// of the chain the warp is advancing.
enum : int { CD_DEPTH, CD_KMIN, CD_DPREV, CD_KPREV, CD_PREV0, CD_PREV1, CD_PREV2, CD_MATCH,
             CD_ENTRY, CD_NMOD, CD_NSKIP, CD_TOTERR, CD_ERRTOT, CD_SERVED, CD_FITTED, CD_COUNT };
enum : int { CI_CHAIN, CI_CUR, CI_END, CI_LEN, CI_TOTLUT, CI_NCOMP, CI_COUNT };
enum : int { CS_HOT, CS_NPREV, CS_ERRCNT, CS_NOPT, CS_ALIVE, CS_COUNT };

struct ChainSmem {
  double d[CD_COUNT][kLutBlock];
  long long i[CI_COUNT][kLutBlock];
  int s[CS_COUNT][kLutBlock];
};

size_t lut_smem_bytes() {
  return sizeof(ChainSmem) + (size_t)kLutBlock * 8 * ((kN + 1) * kN + (kN + 1) + kN);
}

// Ring field k of chain c, slot j: ring[(c * 8 + k) * cap + j]
enum : int { RG_DEPTH, RG_KMIN, RG_RM1, RG_RM2, RG_RM3, RG_PREV0, RG_PREV1, RG_PREV2 };

// model_spectral_diff_mean (model/samodel.c:2792-2842), one region, one
// scene: bands 1..3 below n_bands.
__device__ __forceinline__ float spectral_diff(const double *meas, double l1, double l2,
                                               double l3, int nb) {
  const double lut[3] = {l1, l2, l3};
  double error = 0.0;
  int n_total = 0;
#pragma unroll
  for (int k = 1; k <= 3; k++) {
    if (k >= nb) break;
    double current = 0.0, previous = 0.0, nobs = 0.0;
    if (!((float)meas[k] == 0.0f) && !((float)lut[k - 1] == 0.0f)) {
      current = __dadd_rn(current, meas[k]);
      previous = __dadd_rn(previous, lut[k - 1]);
      nobs = __dadd_rn(nobs, 1.0);
    }
    if (nobs > 0.5) {
      current = current / nobs;
      previous = previous / nobs;
    }
    const double t = __dsub_rn(current, previous) / current;
    error = __dadd_rn(error, __dmul_rn(t, t));
    n_total++;
  }
  error = __dmul_rn(100.0, sqrt(error / (double)n_total));
  return (float)error;
}

// Update of the match and entry thresholds when the slice's 0.1 % count
// moves on (:1182-1211), and the restart of the statistics (:1326-1352).
// Run by the chain's owner lane.
__device__ __forceinline__ void chain_tail(ChainSmem &S, int t, double model_error) {
  const double depth = S.d[CD_DEPTH][t], kmin = S.d[CD_KMIN][t];
  const double dprev = S.d[CD_DPREV][t], kprev = S.d[CD_KPREV][t];
  S.s[CS_HOT][t] = (fabs(__dsub_rn(depth, dprev)) / __dadd_rn(kEps, dprev) < kContinuity &&
                    fabs(__dsub_rn(kmin, kprev)) / __dadd_rn(kEps, kprev) < kContinuity)
                       ? 1
                       : 0;
  S.d[CD_DPREV][t] = depth;
  S.d[CD_KPREV][t] = kmin;
  S.d[CD_TOTERR][t] = __dadd_rn(S.d[CD_TOTERR][t], model_error);
  S.d[CD_NMOD][t] = __dadd_rn(S.d[CD_NMOD][t], 1.0);
  const long long nc = ++S.i[CI_NCOMP][t];
  const int nperc = (int)(__dmul_rn(1000.0, (double)nc) / (double)S.i[CI_LEN][t]);
  if (nperc > S.s[CS_NPREV][t]) {
    double match = S.d[CD_MATCH][t], entry = S.d[CD_ENTRY][t];
    const double n_mod = S.d[CD_NMOD][t];
    if (S.s[CS_NOPT][t] > 0) {
      const int cnt = S.s[CS_ERRCNT][t];
      // vec_mean2_double (model/common.c:877-891) returns a float
      const double error_mean = (double)(float)(cnt ? S.d[CD_ERRTOT][t] / (double)cnt : 0.0);
      match = __dadd_rn(match, __dadd_rn(__dmul_rn(0.75, error_mean),
                                         __dmul_rn(0.25, S.d[CD_TOTERR][t]) / n_mod));
      match = match / 2.0;
      entry = match;
    }
    if (S.d[CD_NSKIP][t] / n_mod > kMaxSkip) {
      match = __dmul_rn(match, 0.75);
      entry = __dmul_rn(entry, 0.75);
    }
    S.d[CD_MATCH][t] = kMinThreshold > match ? kMinThreshold : match;
    S.d[CD_ENTRY][t] = kMinThreshold > entry ? kMinThreshold : entry;
    S.s[CS_NPREV][t] = nperc;
    S.d[CD_TOTERR][t] = 0.0;
    S.d[CD_NMOD][t] = 0.0;
    S.d[CD_NSKIP][t] = 0.0;
    S.s[CS_NOPT][t] = 0;
    S.d[CD_ERRTOT][t] = 0.0;
    S.s[CS_ERRCNT][t] = 0;
  }
  S.i[CI_CUR][t]++;
}

template <int NB>
__global__ void __launch_bounds__(kLutBlock) lut_kernel(const __grid_constant__ LutArgs args) {
  constexpr int BS = kLutBlock;
  const InvertArgs &ia = args.inv;
  const FitParams &fp = ia.fp;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  ChainSmem &S = *reinterpret_cast<ChainSmem *>(smem_raw);
  double *sv = reinterpret_cast<double *>(smem_raw + sizeof(ChainSmem));  // [(N+1)*N][BS]
  double *sf = sv + (kN + 1) * kN * BS;                                     // [N+1][BS]
  double *sbest = sf + (kN + 1) * BS;                                       // [N][BS]

  const int tid = threadIdx.x, lane = tid & 31, wbase = tid & ~31;
  NmLane<kN, P, BS> m;
  m.v = sv + tid;
  m.f = sf + tid;
  double *best = sbest + tid;
  PixelF64<NB> px;
  const double var_limit = P::var_limit(ia);
  const photic_outputs &o = ia.out;
  const int64_t cap = args.cap;

  int64_t pixel = -1;
  int32_t start_k = 0, n_starts = 0, total = 0, kept_evals = 0, kept_start = 0, kept_fault = 0;
  int32_t guard = 0, hot_fit = 0;
  int64_t pending = -1;  // a pixel of this lane's chain waiting for its fit
  double lowest = 0.0;
  bool has = false;
  const int32_t guard_cap = (fp.n_hstarts + 1) * (fp.kcount + 8 * kN + 16);

  S.i[CI_CUR][tid] = 0;
  S.i[CI_END][tid] = 0;  // no chain yet: claim one
  S.s[CS_ALIVE][tid] = 1;
  __syncwarp();

  for (;;) {
    // ---- advance the chains of lanes without a fit in flight -------------
    unsigned need = __ballot_sync(kFull, !has && S.s[CS_ALIVE][tid]);
    while (need) {
      const int L = __ffs(need) - 1, t = wbase + L;
      for (;;) {
        __syncwarp();
        if (S.i[CI_CUR][t] >= S.i[CI_END][t]) {
          // chain finished (or none yet): its tally, then the next chain
          if (lane == L) {
            const long long c_old = S.i[CI_END][t] > 0 ? S.i[CI_CHAIN][t] : -1;
            if (c_old >= 0 && args.chain_stats) {
              double *cs = args.chain_stats + c_old * 4;
              cs[0] = S.d[CD_SERVED][t];
              cs[1] = S.d[CD_FITTED][t];
              cs[2] = S.d[CD_MATCH][t];
              cs[3] = S.d[CD_ENTRY][t];
            }
            const long long c = (long long)atomicAdd(args.queue, 1ull);
            if (c >= args.n_chains) {
              S.s[CS_ALIVE][t] = 0;
              S.i[CI_END][t] = 0;
              S.i[CI_CUR][t] = 0;
            } else {
              const long long a0 = c * args.n_shallow / args.n_chains;
              const long long a1 = (c + 1) * args.n_shallow / args.n_chains;
              S.i[CI_CHAIN][t] = c;
              S.i[CI_CUR][t] = a0;
              S.i[CI_END][t] = a1;
              S.i[CI_LEN][t] = a1 - a0;
              S.i[CI_TOTLUT][t] = 0;
              S.i[CI_NCOMP][t] = 0;
              for (int k = 0; k < CD_COUNT; k++) S.d[k][t] = 0.0;
              S.d[CD_MATCH][t] = kMinThreshold > 1.125 ? kMinThreshold : 1.125;  // :896
              S.d[CD_ENTRY][t] = S.d[CD_MATCH][t];
              S.s[CS_HOT][t] = 0;
              S.s[CS_NPREV][t] = 0;
              S.s[CS_ERRCNT][t] = 0;
              S.s[CS_NOPT][t] = 0;
            }
          }
          __syncwarp();
          if (!S.s[CS_ALIVE][t]) break;
          continue;
        }
        const long long c = S.i[CI_CHAIN][t];
        const int64_t p = args.order[S.i[CI_CUR][t]];
        const float *r = ia.rrs + p * fp.n_bands;
        double meas[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
        for (int b = 1; b < 4; b++)
          if (b < fp.n_bands) meas[b] = (double)__ldg(r + b);
        // lookup (:980-999): the first slot of least difference among the
        // entries continuous with the previous pixel
        const double dep = S.d[CD_DEPTH][t], km = S.d[CD_KMIN][t];
        const long long tl = S.i[CI_TOTLUT][t];
        const int64_t n_in = tl < cap ? tl : cap;
        const double *R = args.ring + (size_t)c * 8 * cap;
        double bestd = 1.0e4;
        int64_t pos = 0;
        for (int64_t j = lane; j < n_in; j += 32) {
          const double de = R[RG_DEPTH * cap + j], ke = R[RG_KMIN * cap + j];
          if (fabs(__dsub_rn(de, dep)) / __dadd_rn(dep, kEps) < kContinuity &&
              fabs(__dsub_rn(ke, km)) / __dadd_rn(km, kEps) < kContinuity) {
            const double d = (double)spectral_diff(meas, R[RG_RM1 * cap + j],
                                                   R[RG_RM2 * cap + j], R[RG_RM3 * cap + j],
                                                   fp.n_bands);
            if (d < bestd) {
              bestd = d;
              pos = j;
            }
          }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
          const double ob = __shfl_xor_sync(kFull, bestd, off);
          const int64_t op = __shfl_xor_sync(kFull, pos, off);
          if (ob < bestd || (ob == bestd && op < pos)) {
            bestd = ob;
            pos = op;
          }
        }
        // (an empty table with a threshold above 1e4 would make the
        // reference serve an unused slot; that pixel is fitted here)
        if (bestd > S.d[CD_MATCH][t] || n_in == 0) {
          // a fit (:1008-1063): set up below, every such lane of the warp
          // at once
          if (lane == L) pending = p;
          break;
        }
        // served (:1066-1073): the entry's outputs, lane k copying field k
        const int64_t src = args.ring_src[(size_t)c * cap + pos];
        switch (lane) {
          case 0: if (o.depth) o.depth[p] = o.depth[src]; break;
          case 1: if (o.depth_f64) o.depth_f64[p] = o.depth_f64[src]; break;
          case 2: if (o.P) o.P[p] = o.P[src]; break;
          case 3: if (o.G) o.G[p] = o.G[src]; break;
          case 4: if (o.X) o.X[p] = o.X[src]; break;
          case 5: if (o.bottom_albedo) o.bottom_albedo[p] = o.bottom_albedo[src]; break;
          case 6: if (o.model_error) o.model_error[p] = (float)bestd; break;
          case 7: if (o.rrs_error) o.rrs_error[p] = o.rrs_error[src]; break;
          case 8: if (o.K_min) o.K_min[p] = o.K_min[src]; break;
          case 9: if (o.iod) o.iod[p] = o.iod[src]; break;
          case 10: if (o.evals) o.evals[p] = 0; break;
          case 11: if (o.evals_kept) o.evals_kept[p] = 0; break;
          case 12:
            if (o.status)
              o.status[p] = PHOTIC_PX_FITTED | PHOTIC_PX_SERVED | (o.status[src] & PHOTIC_PX_CONVERGED);
            break;
          case 13: if (args.source) args.source[p] = src; break;
          default:
            if (lane >= 16 && lane < 22 && o.params) o.params[p * 6 + (lane - 16)] = o.params[src * 6 + (lane - 16)];
            break;
        }
        if (lane == L) {
          S.d[CD_DPREV][t] = S.d[CD_DEPTH][t];
          S.d[CD_KPREV][t] = S.d[CD_KMIN][t];
          S.d[CD_DEPTH][t] = R[RG_DEPTH * cap + pos];
          S.d[CD_KMIN][t] = R[RG_KMIN * cap + pos];
          S.d[CD_PREV0][t] = R[RG_PREV0 * cap + pos];
          S.d[CD_PREV1][t] = R[RG_PREV1 * cap + pos];
          S.d[CD_PREV2][t] = R[RG_PREV2 * cap + pos];
          S.d[CD_NSKIP][t] = __dadd_rn(S.d[CD_NSKIP][t], 1.0);
          S.d[CD_SERVED][t] += 1.0;
          chain_tail(S, t, bestd);
        }
      }
      need &= ~(1u << L);
    }
    if (pending >= 0) {
      const int64_t p = pending;
      const float *r = ia.rrs + p * fp.n_bands;
      pending = -1;
      float rf[NB];
#pragma unroll
      for (int b = 0; b < NB; b++) rf[b] = b < fp.n_bands ? __ldg(r + b) : 0.0f;
      P::template setup<NB>(ia, rf, px);
      pixel = p;
      total = kept_evals = kept_start = kept_fault = guard = 0;
      lowest = 1.0e4;
      start_k = 0;
#pragma unroll
      for (int i = 0; i < kN; i++) best[i * BS] = 0.0;
      P::template cold_start<NB>(ia, px, m.start, m.step);
      // the pixel's empirical depth (:955-979): its single start, hot
      // or cold; a pixel without one is fitted cold
      bool emp_present = false;
      double h_emp = 0.0;
      if (args.emp) {
        const float e = args.emp[p];
        if (!ref_approx_eq(e, args.emp_nodata, 1.0e-6f)) {
          emp_present = true;
          h_emp = (double)e > -1.0 ? 1.0 : fabs((double)e);
        }
      }
      hot_fit = S.s[CS_HOT][tid] && (args.emp == nullptr || emp_present);
      if (hot_fit) {  // :2234-2241, 2285-2305
        const double h = emp_present ? h_emp : S.d[CD_DPREV][tid];
        m.start[0] = h;
        m.step[0] = P::h_step(h);
        m.start[3] = S.d[CD_PREV0][tid];
        m.start[4] = S.d[CD_PREV1][tid];
        m.start[5] = S.d[CD_PREV2][tid];
#pragma unroll
        for (int i = 3; i < 6; i++) m.step[i] = __dmul_rn(2.0, m.start[i]);
        n_starts = 1;
      } else if (emp_present) {  // :2221-2223
        m.start[0] = h_emp;
        m.step[0] = P::h_step(h_emp);
        n_starts = 1;
      } else {
        m.start[0] = P::hstart(ia, 0);
        m.step[0] = P::h_step(m.start[0]);
        n_starts = fp.n_hstarts;
      }
      m.begin(var_limit, fp.konvge, fp.kcount);
      has = true;
    }
    if (!__any_sync(kFull, has)) break;

    // ---- one cost evaluation per lane, then the bookkeeping --------------
    if (has) {
      // one evaluation for every lane; at the kept optimum its kept band
      // values give the products (the final point is evaluated together
      // with the other lanes' trial points)
      BandKeep<NB> keep;
      const double y = P::template cost_keep<NB>(ia, px, m.x, keep);
      if (m.phase == PH_FINAL) {
        typename P::Details det;
        P::template details_from_keep<NB>(ia, keep, y, det);
        const int64_t p = pixel;
        const double H = fabs(m.x[0]);
        if (o.depth) o.depth[p] = (float)H;
        if (o.depth_f64) o.depth_f64[p] = H;
        if (o.P) o.P[p] = (float)(0.01 * fabs(m.x[3]));
        if (o.G) o.G[p] = (float)(0.01 * fabs(m.x[4]));
        if (o.X) o.X[p] = (float)(0.01 * fabs(m.x[5]));
        if (o.bottom_albedo) o.bottom_albedo[p] = (float)det.bottom_albedo;
        if (o.model_error) o.model_error[p] = (float)det.model_error;
        if (o.rrs_error) o.rrs_error[p] = (float)det.rrs_error;
        if (o.K_min) o.K_min[p] = (float)det.K_min;
        if (o.iod) o.iod[p] = (float)det.iod;
        if (o.evals) o.evals[p] = total;
        if (o.evals_kept) o.evals_kept[p] = kept_evals;
        if (o.params)
          for (int i = 0; i < kN; i++) o.params[p * kN + i] = m.x[i];
        if (o.status)
          o.status[p] = PHOTIC_PX_FITTED | (kept_fault == 0 ? PHOTIC_PX_CONVERGED : 0) |
                        (hot_fit ? PHOTIC_PX_HOT : 0) | (kept_start << 16);
        if (args.source) args.source[p] = -1;
        // the chain after a fit (:1027-1063, 1104-1116)
        const double me = det.model_error;
        S.d[CD_DEPTH][tid] = H;
        S.d[CD_KMIN][tid] = det.K_min;
        S.d[CD_PREV0][tid] = fabs(m.x[3]);
        S.d[CD_PREV1][tid] = fabs(m.x[4]);
        S.d[CD_PREV2][tid] = fabs(m.x[5]);
        S.s[CS_NOPT][tid]++;
        if (!((float)me == 0.0f)) {  // vec_mean2_double skips zeros
          S.d[CD_ERRTOT][tid] = __dadd_rn(S.d[CD_ERRTOT][tid], me);
          S.s[CS_ERRCNT][tid]++;
        }
        if (me < S.d[CD_ENTRY][tid] && H < 32.0) {
          const long long c = S.i[CI_CHAIN][tid];
          const long long tl = S.i[CI_TOTLUT][tid];
          const int64_t slot = tl % cap;
          double *R = args.ring + (size_t)c * 8 * cap;
          R[RG_DEPTH * cap + slot] = H;
          R[RG_KMIN * cap + slot] = det.K_min;
          R[RG_RM1 * cap + slot] = fp.n_bands > 1 ? keep.Rm[1] : 0.0;
          R[RG_RM2 * cap + slot] = fp.n_bands > 2 ? keep.Rm[2] : 0.0;
          R[RG_RM3 * cap + slot] = fp.n_bands > 3 ? keep.Rm[3] : 0.0;
          R[RG_PREV0 * cap + slot] = fabs(m.x[3]);
          R[RG_PREV1 * cap + slot] = fabs(m.x[4]);
          R[RG_PREV2 * cap + slot] = fabs(m.x[5]);
          args.ring_src[(size_t)c * cap + slot] = p;
          S.i[CI_TOTLUT][tid] = tl + 1;
        }
        S.d[CD_FITTED][tid] += 1.0;
        chain_tail(S, tid, me);
        has = false;
      } else {
        if (++guard > guard_cap) {
          // Defensive cap: each nelmin call is bounded by kcount, so
          // reaching this means a defect; flag it and drop the chain.
          atomicOr(ia.error, PHOTIC_DEVERR_EVAL_CAP);
          if (o.status) o.status[pixel] = PHOTIC_PX_INVALID;
          S.i[CI_CUR][tid] = S.i[CI_END][tid];
          has = false;
        } else if (m.step_machine(y)) {
          // nelmin returned: keep the best start (model/samodel.c:2380-2405)
          const double ynewlo = m.F(m.lo);
          total += m.icount;
          bool finish = false;
          if (ynewlo < lowest) {
            lowest = ynewlo;
#pragma unroll
            for (int i = 0; i < kN; i++) best[i * BS] = m.xmin[i];
            kept_evals = m.icount;
            kept_start = start_k;
            kept_fault = m.ifault;
            if (lowest < ia.early_exit) finish = true;
          }
          start_k++;
          if (!finish && start_k < n_starts) {
            P::template cold_start<NB>(ia, px, m.start, m.step);
            m.start[0] = P::hstart(ia, start_k);
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

template <int NB>
cudaError_t launch_nb(const LutArgs &a, int grid, cudaStream_t s, int *occupancy) {
  const size_t smem = lut_smem_bytes();
  auto k = lut_kernel<NB>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (occupancy) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occupancy, k, kLutBlock, smem);
  k<<<grid, kLutBlock, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace

int lut_block() { return kLutBlock; }

int lut_blocks_per_sm(const LutArgs &a) {
  int n = 0;
  cudaError_t e = a.inv.fp.n_bands <= 4 ? launch_nb<4>(a, 0, 0, &n) : launch_nb<8>(a, 0, 0, &n);
  return e == cudaSuccess ? n : 0;
}

// The sorted shallow pixels: keys and mask (masked pixels' outputs written
// there), the shallow pixels selected in pixel order, their keys gathered,
// and a stable radix sort of (key, pixel) pairs -- the order of a stable
// sort, which the reference's merge sort gives when no key is NaN; with NaN
// keys, the reference's merge tree over every pixel instead.  order must hold npix
// entries; *n_shallow receives the count (the call synchronises the stream
// once to read it).  Scratch is stream-ordered.
cudaError_t lut_order(LutKeyArgs ka, int64_t *order, int64_t *n_shallow, cudaStream_t s) {
  const int64_t npix = ka.npix;
  *n_shallow = 0;
  if (npix <= 0) return cudaSuccess;
  float *keys = nullptr, *sel_keys = nullptr, *sorted_keys = nullptr;
  uint8_t *flags = nullptr;
  int64_t *idx = nullptr, *sel_idx = nullptr, *d_count = nullptr;
  void *temp = nullptr;
  size_t b_sel = 0, b_sort = 0;
  cudaError_t e = cub::DeviceSelect::Flagged(nullptr, b_sel, idx, flags, sel_idx, d_count, npix, s);
  if (e == cudaSuccess)
    e = cub::DeviceRadixSort::SortPairs(nullptr, b_sort, sel_keys, sorted_keys, sel_idx, order,
                                        npix, 0, 32, s);
  const size_t b_temp = b_sel > b_sort ? b_sel : b_sort;
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&keys, npix * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&sel_keys, npix * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&sorted_keys, npix * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&flags, npix, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&idx, npix * sizeof(int64_t), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&sel_idx, npix * sizeof(int64_t), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_count, sizeof(int64_t), s);
  if (e == cudaSuccess) e = cudaMallocAsync(&temp, b_temp, s);
  if (e == cudaSuccess) {
    ka.keys = keys;
    ka.flags = flags;
    ka.idx = idx;
    const int bs = 256;
    lut_key_kernel<<<(unsigned)((npix + bs - 1) / bs), bs, 0, s>>>(ka);
    e = cudaGetLastError();
  }
  // NaN keys (pixels whose blue, green and red are all nodata or zero,
  // under the spectral-angle order) need the reference's own merge tree
  unsigned long long n_nan = 0;
  if (e == cudaSuccess) e = cudaMemsetAsync(d_count, 0, sizeof(int64_t), s);
  if (e == cudaSuccess) {
    const int bs = 256;
    nan_count_kernel<<<(unsigned)((npix + bs - 1) / bs), bs, 0, s>>>(
        keys, npix, reinterpret_cast<unsigned long long *>(d_count));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&n_nan, d_count, sizeof n_nan, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  int64_t S = 0;
  size_t bt = b_temp;
  if (e == cudaSuccess && n_nan > 0) {
    // merge-sort every pixel's (key, index) level by level, ping-ponging
    // between (keys, idx) and (sorted_keys, sel_idx); then the shallow
    // pixels in that order
    int depth = 0;
    while (((int64_t)1 << depth) < npix) depth++;
    float *ka = keys, *kb = sorted_keys;
    int64_t *ia = idx, *ib = sel_idx;
    for (int d = depth - 1; d >= 0 && e == cudaSuccess; d--) {
      const int64_t nt = (int64_t)1 << d;
      const int bs = 128;
      msort_level_kernel<<<(unsigned)((nt + bs - 1) / bs), bs, 0, s>>>(ka, ia, kb, ib, npix, d);
      e = cudaGetLastError();
      float *tk = ka; ka = kb; kb = tk;
      int64_t *ti = ia; ia = ib; ib = ti;
    }
    uint8_t *sflags = reinterpret_cast<uint8_t *>(kb);  // the free key buffer
    if (e == cudaSuccess) {
      const int bs = 256;
      gather_flags_kernel<<<(unsigned)((npix + bs - 1) / bs), bs, 0, s>>>(flags, ia, npix,
                                                                        sflags);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cub::DeviceSelect::Flagged(temp, bt, ia, sflags, order, d_count, npix, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&S, d_count, sizeof S, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  } else {
    if (e == cudaSuccess)
      e = cub::DeviceSelect::Flagged(temp, bt, idx, flags, sel_idx, d_count, npix, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&S, d_count, sizeof S, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e == cudaSuccess && S > 0 && n_nan == 0) {
    const int bs = 256;
    gather_keys_kernel<<<(unsigned)((S + bs - 1) / bs), bs, 0, s>>>(keys, sel_idx, S, sel_keys);
    e = cudaGetLastError();
    bt = b_temp;
    if (e == cudaSuccess)
      e = cub::DeviceRadixSort::SortPairs(temp, bt, sel_keys, sorted_keys, sel_idx, order, S, 0,
                                          32, s);
  }
  cudaFreeAsync(keys, s);
  cudaFreeAsync(sel_keys, s);
  cudaFreeAsync(sorted_keys, s);
  cudaFreeAsync(flags, s);
  cudaFreeAsync(idx, s);
  cudaFreeAsync(sel_idx, s);
  cudaFreeAsync(d_count, s);
  cudaFreeAsync(temp, s);
  if (e == cudaSuccess) *n_shallow = S;
  return e;
}

cudaError_t launch_lut(const LutArgs &a, int grid, cudaStream_t s) {
  return a.inv.fp.n_bands <= 4 ? launch_nb<4>(a, grid, s, nullptr)
                               : launch_nb<8>(a, grid, s, nullptr);
}

}  // namespace photic
