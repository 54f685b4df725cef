// photic_guarded.cu -- FP64-faithful inversion with double-float screening
// (PHOTIC_PREC_GUARDED).
//
// GB300 runs FP64 at 1/58 of its FP32 warp-instruction rate, and an FP64
// instruction costs the same pipe time whether 1 or 32 lanes are active.
// The Nelder-Mead trajectory of the reference (model/asa047.c:10-502)
// depends on the costs only through comparisons, the variance test and the
// (long)(10*y) local-minimum test.  So:
//   * vertex coordinates and all simplex bookkeeping stay in IEEE double in
//     the reference's operation order (bit-identical points);
//   * every cost is first evaluated in double-float (~48 bits, FP32 pipes);
//   * a decision is taken on the double-float values when their gap exceeds
//     kTau times their magnitude (the double-float cost agrees with the
//     double one to ~1e-14); otherwise the exact double-precision cost of the
//     undecided value is requested.  On this workload about 1 % of
//     comparisons are that close;
//   * requests are posted to a block-wide ring in shared memory and served
//     32 at a time by whichever warp finds the ring full enough (or all of
//     its own lanes waiting), so the FP64 cost runs with full warps.
// The decisions, and hence the trajectory, are those of the FP64 kernel.
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_dfcost.cuh"
#include "photic_fp64.cuh"
#include "photic_kernels.h"

namespace photic {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kN = 6;
// Relative gap below which a double-float comparison is deferred to FP64.
constexpr float kTau = 1.0e-11f;

// Value slots that can be re-evaluated exactly.
enum : int32_t { SL_REFL = kN + 1, SL_TRIAL, SL_PROBE, SL_BEST, SL_NONE = -1 };

enum : int32_t {
  PHX_INIT_BASE = 0,
  PHX_INIT_VERT,
  PHX_REFLECT,
  PHX_EXPAND,
  PHX_CONTRACT_IN,
  PHX_CONTRACT_OUT,
  PHX_SHRINK,
  PHX_PROBE_PLUS,
  PHX_PROBE_MINUS,
  PHX_FINAL,
  PHX_WAIT
};

enum : int32_t {
  CX_NONE = -1,
  CX_READY = 0,
  CX_TOP,
  CX_DEC_REFLECT,
  CX_DEC_EXPAND,
  CX_DEC_CIN,
  CX_DEC_COUT,
  CX_ITER_END,
  CX_VARTEST,
  CX_END_INNER,
  CX_PROBE_PLUS,
  CX_DEC_PROBE_PLUS,
  CX_DEC_PROBE_MINUS,
  CX_PROBE_END,
  CX_NM_DONE,
  CX_NM_DONE2
};

// A cost value known in double-float and possibly exactly.
struct Lv {
  df64 df;
  double ex;
  bool has;
};

__device__ __forceinline__ float dabs_hi(df64 a) { return fabsf(a.hi); }

// The double-float cost differs from the double one by a relative part
// (~1e-14) and an absolute part from the residuals Rm - Rs, whose rounding
// is relative to Rm rather than to the (possibly tiny) misfit: about
// 2^-44 * 100 * max(Rs) / mean(Rs) in cost units.  kTau and tol_abs keep a
// factor >= 10 over both.
__device__ __forceinline__ float screen_tol(const Lv &a, const Lv &b, float tol_abs) {
  return kTau * (dabs_hi(a.df) + dabs_hi(b.df)) + tol_abs;
}

// Per-lane tally of how decisions were taken (photic_set_guard_stats):
// on exact values already known, on the double-float screen, or deferred to
// an exact FP64 evaluation.
struct Tally {
  unsigned long long exact, screened, deferred;
};

// a < b decided on double-float values when the gap is clear of the
// screening tolerance; returns 0/1, or 2 when exact values are needed.
__device__ __forceinline__ int lz_lt(const Lv &a, const Lv &b, float tol_abs, Tally &t) {
  if (a.has && b.has) {
    t.exact++;
    return a.ex < b.ex;
  }
  df64 d = df_sub(a.df, b.df);
  if (fabsf(d.hi) > screen_tol(a, b, tol_abs)) {
    t.screened++;
    return d.hi < 0.0f;
  }
  t.deferred++;
  return 2;
}
__device__ __forceinline__ int lz_le(const Lv &a, const Lv &b, float tol_abs, Tally &t) {
  if (a.has && b.has) {
    t.exact++;
    return a.ex <= b.ex;
  }
  df64 d = df_sub(a.df, b.df);
  if (fabsf(d.hi) > screen_tol(a, b, tol_abs)) {
    t.screened++;
    return d.hi < 0.0f;
  }
  t.deferred++;
  return 2;
}

// trunc((long)(10*y)) from a double-float value when no integer lies within
// the screening tolerance of 10*y; sets *ok = false otherwise.
__device__ __forceinline__ long long lz_trunc10(const Lv &a, bool *ok, float tol_abs,
                                                Tally &t) {
  if (a.has) {
    t.exact++;
    *ok = true;
    return trunc10(a.ex);
  }
  df64 w = df_mul_f(a.df, 10.0f);
  float r = rintf(w.hi);
  df64 dist = df_add_f(w, -r);
  float tol = 10.0f * (kTau * dabs_hi(a.df) + tol_abs);
  if (!(fabsf(dist.hi) > tol) || !(fabsf(w.hi) < 1.0e15f)) {
    t.deferred++;
    *ok = false;
    return 0;
  }
  t.screened++;
  *ok = true;
  return df_trunc10(a.df);
}

template <int NB, int BS>
struct Shared {
  double v[(kN + 1) * kN][BS];   // vertex coordinates
  double fex[kN + 1][BS];        // exact vertex costs (valid where the mask bit is set)
  df64 fdf[kN + 1][BS];          // double-float vertex costs
  double best[kN][BS];
  double rq_x[kN][BS];           // exact-evaluation request point
  double rq_y[BS];               // its cost
  double px_rrs[NB][BS], px_pw[NB][BS], px_mean[BS];  // FP64 pixel constants
  int32_t rq_state[BS];          // 0 idle, 1 posted, 2 served
  int32_t ring[BS];              // requesting thread + 1, 0 = empty
  int32_t ring_head, ring_tail, lock;
  unsigned long long served;     // exact evaluations served by this block
  unsigned long long stats[5];   // exact, screened, deferred decisions; wait and busy trips
  float chunk[BS / 32][32][NB];
};

template <int NB, int BS>
__global__ void __launch_bounds__(BS) guarded_kernel(const __grid_constant__ InvertArgs args) {
  const FitParams &fp = args.fp;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Shared<NB, BS> &S = *reinterpret_cast<Shared<NB, BS> *>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  if (tid == 0) {
    S.ring_head = 0;
    S.ring_tail = 0;
    S.lock = 0;
    S.served = 0;
    for (int i = 0; i < 5; i++) S.stats[i] = 0;
  }
  S.ring[tid] = 0;
  S.rq_state[tid] = 0;
  __syncthreads();

  const photic_outputs &o = args.out;
  const double var_limit = fp.reqmin * (double)kN;
  Tally tally = {0ull, 0ull, 0ull};
  unsigned long long wait_trips = 0, busy_trips = 0;

  // ---- per-lane state ----------------------------------------------------
  PixelDF<NB> pd;
  double cen[kN], refl[kN], trial[kN], xmin[kN], start[kN], step[kN];
  df64 xe[kN];  // point of the next double-float evaluation
  Lv fr, ft, fpb, ylo, lowest;
  int32_t ylo_src = 0, exmask = 0;
  double scale = 1.0;
  long long floor_lo = 0;
  int32_t phase = PHX_INIT_BASE, cs_resume = CX_NONE, jj = 0, hi = 0, lo = 0;
  int32_t icount = 0, numres = 0, ifault = 0, countdown = 0;
  int32_t req_slot = SL_NONE, wait_age = 0;
  int64_t pixel = -1;
  int32_t start_k = 0, n_starts = 0, total = 0, kept_evals = 0, kept_start = 0, kept_fault = 0;
  int32_t guard = 0;
  float tol_abs = 0.0f;
  bool has = false, open = true, retired = false;
  int64_t chunk_base = 0, chunk_next = 0, chunk_end = 0;
  const int32_t guard_cap = 4 * (fp.n_hstarts + 1) * (fp.kcount + 8 * kN + 16);

  auto V = [&](int j, int i) -> double & { return S.v[j * kN + i][tid]; };
  auto Fv = [&](int j) -> Lv {
    Lv r;
    r.df = S.fdf[j][tid];
    r.ex = S.fex[j][tid];
    r.has = (exmask >> j) & 1;
    return r;
  };
  auto setF = [&](int j, const Lv &val) {
    S.fdf[j][tid] = val.df;
    S.fex[j][tid] = val.ex;
    exmask = (exmask & ~(1 << j)) | (val.has ? (1 << j) : 0);
  };
  auto lv_df = [](df64 d) {
    Lv r;
    r.df = d;
    r.ex = 0.0;
    r.has = false;
    return r;
  };
  auto set_eval = [&](const double *p) {
#pragma unroll
    for (int i = 0; i < kN; i++) xe[i] = df_from_double(p[i]);
  };
  auto post = [&](int slot, const double *p) {
#pragma unroll
    for (int i = 0; i < kN; i++) S.rq_x[i][tid] = p[i];
    req_slot = slot;
    S.rq_state[tid] = 1;
    __threadfence_block();
    const int at = atomicAdd(&S.ring_tail, 1);
    atomicExch(&S.ring[at % BS], tid + 1);
    wait_age = 0;
    phase = PHX_WAIT;
  };
  // Request the exact cost of value slot s (vertex j, or a named point).
  auto need = [&](int s) {
    double p[kN];
    if (s <= kN) {
#pragma unroll
      for (int i = 0; i < kN; i++) p[i] = V(s, i);
    } else if (s == SL_REFL) {
#pragma unroll
      for (int i = 0; i < kN; i++) p[i] = refl[i];
    } else if (s == SL_TRIAL) {
#pragma unroll
      for (int i = 0; i < kN; i++) p[i] = trial[i];
    } else if (s == SL_PROBE) {
#pragma unroll
      for (int i = 0; i < kN; i++) p[i] = xmin[i];
    } else {
#pragma unroll
      for (int i = 0; i < kN; i++) p[i] = S.best[i][tid];
    }
    post(s, p);
  };
  // First slot of a comparison that lacks its exact value.
  auto pick_need = [&](const Lv &a, int sa, const Lv &b, int sb) { return !a.has ? sa : sb; };
  auto make_vertex = [&](int j) {
    double p[kN];
#pragma unroll
    for (int i = 0; i < kN; i++) {
      double s = start[i];
      if (i == j) s = start[i] + step[i] * scale;
      p[i] = s;
      V(j, i) = s;
    }
    set_eval(p);
    jj = j;
    phase = PHX_INIT_VERT;
  };
  auto restart_simplex = [&]() {
#pragma unroll
    for (int i = 0; i < kN; i++) V(kN, i) = start[i];
    set_eval(start);
    phase = PHX_INIT_BASE;
  };
  auto begin = [&]() {
    countdown = fp.konvge;
    icount = 0;
    numres = 0;
    ifault = 0;
    scale = 1.0;
    exmask = 0;
    restart_simplex();
  };
  auto start_cold = [&](int k) {
    double h = fp.hstarts[0];
    for (int i = 1; i < kMaxHStarts; i++)
      if (i == k) h = fp.hstarts[i];
    PixelF64<NB> pf;
#pragma unroll
    for (int b = 0; b < NB; b++) {
      pf.rrs[b] = S.px_rrs[b][tid];
      pf.pw[b] = S.px_pw[b][tid];
    }
    pf.mean = S.px_mean[tid];
    pf.r490 = 0.0;
    pf.r550 = 0.0;
    pf.r640 = 0.0;
    // r490/r550/r640 from the measured spectrum (model/samodel.c:1785-1799)
    pf.r490 = interp_plan<NB>(fp.plan[1], pf.rrs);
    pf.r550 = interp_plan<NB>(fp.plan[2], pf.rrs);
    pf.r640 = interp_plan<NB>(fp.plan[3], pf.rrs);
    cold_start_f64<NB>(fp, pf, start, step);
    start[0] = h;
    step[0] = 1.25 * start[0];
  };
  // Overwriting vertex j would lose the point behind ylo's exact value.
  auto guard_overwrite = [&](int j) -> bool {
    if (j == ylo_src && !ylo.has && !((exmask >> j) & 1)) {
      need(j);
      return true;
    }
    if (j == ylo_src && !ylo.has) {  // vertex already exact: take it
      ylo.ex = S.fex[j][tid];
      ylo.has = true;
    }
    return false;
  };
  auto replace_hi = [&](const double *p, const Lv &val) {
#pragma unroll
    for (int i = 0; i < kN; i++) V(hi, i) = p[i];
    setF(hi, val);
  };

  // Run the machine until it needs a double-float evaluation (returns 0), an
  // exact evaluation (1, request posted), or the pixel is done (2).
  auto run = [&](int cs) -> int {
    while (true) {
      switch (cs) {
        case CX_READY: {  // argmin (model/asa047.c:200-210)
          Lv best_v = Fv(0);
          int bl = 0;
          for (int j = 1; j <= kN; j++) {
            Lv fj = Fv(j);
            int r = lz_lt(fj, best_v, tol_abs, tally);
            if (r == 2) {
              cs_resume = CX_READY;
              need(pick_need(fj, j, best_v, bl));
              return 1;
            }
            if (r) {
              best_v = fj;
              bl = j;
            }
          }
          ylo = best_v;
          ylo_src = bl;
          lo = bl;
          cs = CX_TOP;
          break;
        }
        case CX_TOP: {  // model/asa047.c:213-250
          if (fp.kcount <= icount) {
            cs = CX_END_INNER;
            break;
          }
          Lv yhi = Fv(0);
          int h = 0;
          for (int j = 1; j <= kN; j++) {
            Lv fj = Fv(j);
            int r = lz_lt(yhi, fj, tol_abs, tally);
            if (r == 2) {
              cs_resume = CX_TOP;
              need(pick_need(yhi, h, fj, j));
              return 1;
            }
            if (r) {
              yhi = fj;
              h = j;
            }
          }
          hi = h;
#pragma unroll
          for (int i = 0; i < kN; i++) {
            double z = 0.0;
#pragma unroll
            for (int j = 0; j <= kN; j++) z = z + V(j, i);
            z = z - V(hi, i);
            cen[i] = fm::div_by(z, (double)kN, 1.0 / (double)kN);
          }
#pragma unroll
          for (int i = 0; i < kN; i++) refl[i] = cen[i] + (cen[i] - V(hi, i));
          set_eval(refl);
          phase = PHX_REFLECT;
          return 0;
        }
        case CX_DEC_REFLECT: {  // model/asa047.c:251-329
          int r = lz_lt(fr, ylo, tol_abs, tally);
          if (r == 2) {
            cs_resume = CX_DEC_REFLECT;
            need(pick_need(fr, SL_REFL, ylo, ylo_src));
            return 1;
          }
          if (r) {
#pragma unroll
            for (int i = 0; i < kN; i++) trial[i] = cen[i] + 2.0 * (refl[i] - cen[i]);
            set_eval(trial);
            phase = PHX_EXPAND;
            return 0;
          }
          int worse = 0;
          for (int j = 0; j <= kN; j++) {
            Lv fj = Fv(j);
            int q = lz_lt(fr, fj, tol_abs, tally);
            if (q == 2) {
              cs_resume = CX_DEC_REFLECT;
              need(pick_need(fr, SL_REFL, fj, j));
              return 1;
            }
            worse += q;
          }
          if (worse > 1) {
            if (guard_overwrite(hi)) {
              cs_resume = CX_DEC_REFLECT;
              return 1;
            }
            replace_hi(refl, fr);
            cs = CX_ITER_END;
          } else if (worse == 0) {
#pragma unroll
            for (int i = 0; i < kN; i++) trial[i] = cen[i] + 0.5 * (V(hi, i) - cen[i]);
            set_eval(trial);
            phase = PHX_CONTRACT_IN;
            return 0;
          } else {
#pragma unroll
            for (int i = 0; i < kN; i++) trial[i] = cen[i] + 0.5 * (refl[i] - cen[i]);
            set_eval(trial);
            phase = PHX_CONTRACT_OUT;
            return 0;
          }
          break;
        }
        case CX_DEC_EXPAND: {
          int r = lz_lt(fr, ft, tol_abs, tally);
          if (r == 2) {
            cs_resume = CX_DEC_EXPAND;
            need(pick_need(fr, SL_REFL, ft, SL_TRIAL));
            return 1;
          }
          if (guard_overwrite(hi)) {
            cs_resume = CX_DEC_EXPAND;
            return 1;
          }
          if (r) replace_hi(refl, fr);
          else replace_hi(trial, ft);
          cs = CX_ITER_END;
          break;
        }
        case CX_DEC_CIN: {
          Lv fh = Fv(hi);
          int r = lz_lt(fh, ft, tol_abs, tally);
          if (r == 2) {
            cs_resume = CX_DEC_CIN;
            need(pick_need(fh, hi, ft, SL_TRIAL));
            return 1;
          }
          if (r) {
            // shrink towards the best vertex (model/asa047.c:331-351); every
            // vertex is rewritten, so ylo is re-derived afterwards
#pragma unroll
            for (int i = 0; i < kN; i++) {
              double s = (V(0, i) + V(lo, i)) * 0.5;
              V(0, i) = s;
              xmin[i] = s;
            }
            set_eval(xmin);
            jj = 0;
            phase = PHX_SHRINK;
            return 0;
          }
          if (guard_overwrite(hi)) {
            cs_resume = CX_DEC_CIN;
            return 1;
          }
          replace_hi(trial, ft);
          cs = CX_ITER_END;
          break;
        }
        case CX_DEC_COUT: {
          int r = lz_le(ft, fr, tol_abs, tally);
          if (r == 2) {
            cs_resume = CX_DEC_COUT;
            need(pick_need(ft, SL_TRIAL, fr, SL_REFL));
            return 1;
          }
          if (guard_overwrite(hi)) {
            cs_resume = CX_DEC_COUT;
            return 1;
          }
          if (r) replace_hi(trial, ft);
          else replace_hi(refl, fr);
          cs = CX_ITER_END;
          break;
        }
        case CX_ITER_END: {  // model/asa047.c:395-405
          Lv fh = Fv(hi);
          int r = lz_lt(fh, ylo, tol_abs, tally);
          if (r == 2) {
            cs_resume = CX_ITER_END;
            need(pick_need(fh, hi, ylo, ylo_src));
            return 1;
          }
          if (r) {
            ylo = fh;
            ylo_src = hi;
            lo = hi;
          }
          countdown--;
          cs = countdown > 0 ? CX_TOP : CX_VARTEST;
          break;
        }
        case CX_VARTEST: {  // model/asa047.c:406-434
          if (!(icount <= fp.kcount)) {
            cs = CX_TOP;
            break;
          }
          // screen on double-float values
          df64 z = df64{0.0f, 0.0f};
          float amax = 0.0f;
          for (int j = 0; j <= kN; j++) {
            df64 fj = S.fdf[j][tid];
            z = df_add(z, fj);
            amax = fmaxf(amax, fabsf(fj.hi));
          }
          df64 mean = df_div_f(z, (float)(kN + 1));
          z = df64{0.0f, 0.0f};
          float sabs = 0.0f;
          for (int j = 0; j <= kN; j++) {
            df64 d = df_sub(S.fdf[j][tid], mean);
            z = df_add(z, df_mul(d, d));
            sabs += fabsf(d.hi);
          }
          const df64 lim = df_from_double(var_limit);
          df64 gap = df_sub(z, lim);
          float bound = 8.0f * (kTau * amax + tol_abs) * sabs + 8.0f * tol_abs * tol_abs +
                1.0e-12f * fabsf(lim.hi);
          bool all_exact = exmask == (1 << (kN + 1)) - 1;
          bool pass;
          if (!all_exact && fabsf(gap.hi) > bound) {
            pass = gap.hi <= 0.0f;
          } else if (!all_exact) {
            int j = 0;
            while ((exmask >> j) & 1) j++;
            cs_resume = CX_VARTEST;
            need(j);
            return 1;
          } else {
            double zz = 0.0;
            for (int j = 0; j <= kN; j++) zz = zz + S.fex[j][tid];
            double xm = fm::div_by(zz, (double)(kN + 1), 1.0 / (double)(kN + 1));
            zz = 0.0;
            for (int j = 0; j <= kN; j++) {
              double d = S.fex[j][tid] - xm;
              zz = zz + d * d;
            }
            pass = zz <= var_limit;
          }
          countdown = fp.konvge;
          cs = pass ? CX_END_INNER : CX_TOP;
          break;
        }
        case CX_END_INNER: {  // model/asa047.c:436-453
          Lv fl = Fv(lo);
          bool ok;
          long long f10 = lz_trunc10(fl, &ok, tol_abs, tally);
          if (!ok) {
            cs_resume = CX_END_INNER;
            need(lo);
            return 1;
          }
#pragma unroll
          for (int i = 0; i < kN; i++) xmin[i] = V(lo, i);
          floor_lo = f10;
          if (fp.kcount < icount) {
            ifault = 2;
            cs = CX_NM_DONE;
          } else {
            ifault = 0;
            jj = 0;
            cs = CX_PROBE_PLUS;
          }
          break;
        }
        case CX_PROBE_PLUS: {
          double del = step[0] * 1.0e-6;
#pragma unroll
          for (int i = 1; i < kN; i++)
            if (i == jj) del = step[i] * 1.0e-6;
#pragma unroll
          for (int i = 0; i < kN; i++)
            if (i == jj) xmin[i] = xmin[i] + del;
          set_eval(xmin);
          phase = PHX_PROBE_PLUS;
          return 0;
        }
        case CX_DEC_PROBE_PLUS:
        case CX_DEC_PROBE_MINUS: {
          bool ok;
          long long t = lz_trunc10(fpb, &ok, tol_abs, tally);
          if (!ok) {
            cs_resume = cs;
            need(SL_PROBE);
            return 1;
          }
          if (t < floor_lo) {
            ifault = 2;
            cs = CX_PROBE_END;
            break;
          }
          double del = step[0] * 1.0e-6;
#pragma unroll
          for (int i = 1; i < kN; i++)
            if (i == jj) del = step[i] * 1.0e-6;
          if (cs == CX_DEC_PROBE_PLUS) {
#pragma unroll
            for (int i = 0; i < kN; i++)
              if (i == jj) xmin[i] = xmin[i] - del - del;
            set_eval(xmin);
            phase = PHX_PROBE_MINUS;
            return 0;
          }
#pragma unroll
          for (int i = 0; i < kN; i++)
            if (i == jj) xmin[i] = xmin[i] + del;
          jj++;
          cs = (jj < kN) ? CX_PROBE_PLUS : CX_PROBE_END;
          break;
        }
        case CX_PROBE_END:
          if (ifault == 0) {
            cs = CX_NM_DONE;
          } else {
#pragma unroll
            for (int i = 0; i < kN; i++) start[i] = xmin[i];
            scale = 1.0e-6;
            numres++;
            restart_simplex();
            return 0;
          }
          break;
        case CX_NM_DONE: {  // model/samodel.c:2380-2405
          Lv yn = Fv(lo);
          int r = lz_lt(yn, lowest, tol_abs, tally);
          if (r == 2) {
            cs_resume = CX_NM_DONE;
            need(pick_need(yn, lo, lowest, SL_BEST));
            return 1;
          }
          if (r && !yn.has) {  // keep the kept cost exact (its point is V(lo))
            cs_resume = CX_NM_DONE;
            need(lo);
            return 1;
          }
          total += icount;
          if (r) {
            lowest = yn;
#pragma unroll
            for (int i = 0; i < kN; i++) S.best[i][tid] = xmin[i];
            kept_evals = icount;
            kept_start = start_k;
            kept_fault = ifault;
            cs = CX_NM_DONE2;
          } else {
            start_k++;
            if (start_k < n_starts) {
              start_cold(start_k);
              begin();
              return 0;
            }
            phase = PHX_FINAL;
            return 2;
          }
          break;
        }
        case CX_NM_DONE2: {  // early exit test on the kept cost
          Lv ee;
          ee.df = df_from_double(args.early_exit);
          ee.ex = args.early_exit;
          ee.has = true;
          int r = lz_lt(lowest, ee, tol_abs, tally);
          if (r == 2) {
            cs_resume = CX_NM_DONE2;
            need(SL_BEST);
            return 1;
          }
          start_k++;
          if (!r && start_k < n_starts) {
            start_cold(start_k);
            begin();
            return 0;
          }
          phase = PHX_FINAL;
          return 2;
        }
        default:
          return 0;
      }
    }
  };

  // Deliver an exact value to its slot.
  auto deliver = [&](double y) {
    const int s = req_slot;
    if (s >= 0 && s <= kN) {
      S.fex[s][tid] = y;
      exmask |= 1 << s;
      if (s == ylo_src && !ylo.has) {
        ylo.ex = y;
        ylo.has = true;
      }
    } else if (s == SL_REFL) {
      fr.ex = y;
      fr.has = true;
    } else if (s == SL_TRIAL) {
      ft.ex = y;
      ft.has = true;
    } else if (s == SL_PROBE) {
      fpb.ex = y;
      fpb.has = true;
    } else if (s == SL_BEST) {
      lowest.ex = y;
      lowest.has = true;
    }
    req_slot = SL_NONE;
  };

  for (;;) {
    // ---- hand out pixels ---------------------------------------------------
    unsigned needp = __ballot_sync(kFull, !has && open && !retired);
    while (needp) {
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
        const int64_t p = chunk_base + lane;
        if (p < args.npix) {
          if (NB == 4 && args.vec4) {
            const float4 v4 = __ldg(reinterpret_cast<const float4 *>(args.rrs) + p);
            S.chunk[warp][lane][0] = v4.x;
            S.chunk[warp][lane][1] = v4.y;
            S.chunk[warp][lane][2] = v4.z;
            S.chunk[warp][lane][3 % NB] = v4.w;
          } else {
#pragma unroll
            for (int b = 0; b < NB; b++)
              S.chunk[warp][lane][b] =
                  b < fp.n_bands ? __ldg(args.rrs + p * args.pixel_stride + b * args.band_stride)
                                 : 0.0f;
          }
        }
        __syncwarp();
      }
      const int rank = __popc(needp & lt_mask);
      const int avail = (int)(chunk_end - chunk_next);
      const bool mine = ((needp >> lane) & 1u) && rank < avail;
      const unsigned taken = __ballot_sync(kFull, mine);
      bool masked = false;
      if (mine) {
        const int64_t p = chunk_next + rank;
        float r[NB];
#pragma unroll
        for (int b = 0; b < NB; b++) r[b] = S.chunk[warp][(int)(p - chunk_base)][b];
#pragma unroll
        for (int b = 0; b < NB; b++)
          if (b < fp.n_bands) {
            float diff = __fsub_rn(r[b], fp.nodata);
            double big = fabs((double)r[b]) < fabs((double)fp.nodata) ? fabs((double)fp.nodata)
                                                                       : fabs((double)r[b]);
            if (fabs((double)diff) <= big * (double)1.0e-6f || r[b] < 0.0f) masked = true;
          }
        if (masked) {
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
            for (int i = 0; i < kN; i++) o.params[p * kN + i] = 0.0;
        } else {
          // FP64 pixel constants (shared, for exact evaluations) and the
          // double-float ones (registers, for screening)
          double rd[NB];
#pragma unroll
          for (int b = 0; b < NB; b++) rd[b] = (double)r[b];
          PixelF64<NB> pf;
          pixel_setup_f64<NB>(fp, args.sc, rd, pf);
#pragma unroll
          for (int b = 0; b < NB; b++) {
            S.px_rrs[b][tid] = pf.rrs[b];
            S.px_pw[b][tid] = pf.pw[b];
          }
          S.px_mean[tid] = pf.mean;
          {
            float rmax = 0.0f;
#pragma unroll
            for (int b = 0; b < NB; b++)
              if (b < fp.n_bands) rmax = fmaxf(rmax, fabsf(r[b]));
            tol_abs = 4.0e-13f * 100.0f * rmax / (float)pf.mean + 1.0e-30f;
          }
          pixel_setup_df<NB>(fp, args.ds, r, pd);
          pixel = p;
          total = kept_evals = kept_start = kept_fault = guard = 0;
          lowest.df = df64{1.0e4f, 0.0f};
          lowest.ex = 1.0e4;
          lowest.has = true;
          start_k = 0;
          bool seeded = false;
#pragma unroll
          for (int i = 0; i < kN; i++) S.best[i][tid] = 0.0;
          if (args.seeds != nullptr) {
            const double *sd = args.seeds + p * kN;
            if (!isnan(sd[0])) {
              const double rel[kN] = {1.25, 1.5, 0.5, 2.0, 2.0, 2.0};
              seeded = true;
#pragma unroll
              for (int i = 0; i < kN; i++) {
                start[i] = sd[i];
                step[i] = (rel[i] * fp.seed_step_scale) * sd[i];
              }
            }
          }
          n_starts = seeded ? 1 : fp.n_hstarts;
          if (!seeded) start_cold(0);
          begin();
          has = true;
        }
      }
      chunk_next += __popc(taken);
      needp &= ~taken;
      needp |= __ballot_sync(kFull, mine && masked);
    }
    if (!__any_sync(kFull, has)) break;

    // ---- one double-float evaluation per lane, then the bookkeeping --------
    if (has) {
      busy_trips++;
      if (phase == PHX_WAIT) wait_trips++;
      if (phase == PHX_WAIT) {
        if (*((volatile int32_t *)&S.rq_state[tid]) == 2) {
          __threadfence_block();
          const double y = S.rq_y[tid];
          S.rq_state[tid] = 0;
          deliver(y);
          const int rr = run(cs_resume);
          if (rr == 2) phase = PHX_FINAL;
        } else {
          wait_age++;
        }
      } else if (phase != PHX_FINAL) {
        const df64 y = cost_df<false, NB>(fp, args.ds, pd, xe, nullptr);
        int cs = CX_NONE;
        switch (phase) {
          case PHX_INIT_BASE:
            setF(kN, lv_df(y));
            icount++;
            make_vertex(0);
            break;
          case PHX_INIT_VERT:
            setF(jj, lv_df(y));
            icount++;
            if (jj + 1 < kN) make_vertex(jj + 1);
            else cs = CX_READY;
            break;
          case PHX_REFLECT:
            fr = lv_df(y);
            icount++;
            cs = CX_DEC_REFLECT;
            break;
          case PHX_EXPAND:
            ft = lv_df(y);
            icount++;
            cs = CX_DEC_EXPAND;
            break;
          case PHX_CONTRACT_IN:
            ft = lv_df(y);
            icount++;
            cs = CX_DEC_CIN;
            break;
          case PHX_CONTRACT_OUT:
            ft = lv_df(y);
            icount++;
            cs = CX_DEC_COUT;
            break;
          case PHX_SHRINK:
            setF(jj, lv_df(y));
            icount++;
            if (jj < kN) {
              const int j = jj + 1;
              double p[kN];
#pragma unroll
              for (int i = 0; i < kN; i++) {
                double s = (V(j, i) + V(lo, i)) * 0.5;
                V(j, i) = s;
                p[i] = s;
              }
              set_eval(p);
              jj = j;
            } else {
              cs = CX_READY;
            }
            break;
          case PHX_PROBE_PLUS:
            fpb = lv_df(y);
            icount++;
            cs = CX_DEC_PROBE_PLUS;
            break;
          case PHX_PROBE_MINUS:
            fpb = lv_df(y);
            icount++;
            cs = CX_DEC_PROBE_MINUS;
            break;
          default:
            break;
        }
        if (cs != CX_NONE) {
          const int rr = run(cs);
          if (rr == 2) phase = PHX_FINAL;
        }
      }
      if (++guard > guard_cap) {
        atomicOr(args.error, PHOTIC_DEVERR_EVAL_CAP);
        if (o.status) o.status[pixel] = PHOTIC_PX_INVALID;
        has = false;
        retired = true;  // its request, if any, may still be in the ring
      }
    }

    // ---- final products in FP64 (one per finished pixel) -------------------
    if (has && phase == PHX_FINAL) {
      PixelF64<NB> pf;
#pragma unroll
      for (int b = 0; b < NB; b++) {
        pf.rrs[b] = S.px_rrs[b][tid];
        pf.pw[b] = S.px_pw[b][tid];
      }
      pf.mean = S.px_mean[tid];
      pf.r490 = pf.r550 = pf.r640 = 0.0;
      double xb[kN];
#pragma unroll
      for (int i = 0; i < kN; i++) xb[i] = S.best[i][tid];
      CostDetailsF64 det;
      cost_f64<true, NB>(fp, args.sc, pf, xb, &det);
      const int64_t p = pixel;
      const double H = fabs(xb[0]);
      if (o.depth) o.depth[p] = (float)H;
      if (o.depth_f64) o.depth_f64[p] = H;
      if (o.P) o.P[p] = (float)(0.01 * fabs(xb[3]));
      if (o.G) o.G[p] = (float)(0.01 * fabs(xb[4]));
      if (o.X) o.X[p] = (float)(0.01 * fabs(xb[5]));
      if (o.bottom_albedo) o.bottom_albedo[p] = (float)det.bottom_albedo;
      if (o.model_error) o.model_error[p] = (float)det.model_error;
      if (o.rrs_error) o.rrs_error[p] = (float)det.rrs_error;
      if (o.K_min) o.K_min[p] = (float)det.K_min;
      if (o.iod) o.iod[p] = (float)det.iod;
      if (o.evals) o.evals[p] = total;
      if (o.evals_kept) o.evals_kept[p] = kept_evals;
      if (o.params)
        for (int i = 0; i < kN; i++) o.params[p * kN + i] = xb[i];
      if (o.status)
        o.status[p] = PHOTIC_PX_FITTED | (kept_fault == 0 ? PHOTIC_PX_CONVERGED : 0) |
                      (kept_start << 16);
      has = false;
    }

    // ---- serve exact-evaluation requests, 32 per warp pass -----------------
    {
      const int pending = *((volatile int32_t *)&S.ring_tail) - *((volatile int32_t *)&S.ring_head);
      const bool mine_wait = has && phase == PHX_WAIT;
      const unsigned waiting = __ballot_sync(kFull, mine_wait);
      const unsigned active = __ballot_sync(kFull, has);
      const bool old = __any_sync(kFull, mine_wait && wait_age >= 4);
      const bool go = pending >= 32 || (pending > 0 && (waiting == active || old || !open));
      if (go) {
        int got = 0;
        if (lane == 0) got = atomicCAS(&S.lock, 0, 1) == 0;
        got = __shfl_sync(kFull, got, 0);
        if (got) {
          __threadfence_block();
          const int h = *((volatile int32_t *)&S.ring_head);
          const int t = *((volatile int32_t *)&S.ring_tail);
          const int n = min(32, t - h);
          int e = 0;
          if (lane < n) e = *((volatile int32_t *)&S.ring[(h + lane) % BS]);
          // take the leading run of entries that are already written
          const unsigned ready = __ballot_sync(kFull, lane < n && e != 0);
          const int nr = ready == kFull ? 32 : __ffs(~ready) - 1;
          const bool serve = lane < nr;
          if (serve) S.ring[(h + lane) % BS] = 0;
          __syncwarp();
          if (lane == 0) {
            S.ring_head = h + nr;
            S.served += (unsigned long long)nr;
          }
          if (serve) {
            const int L = e - 1;
            PixelF64<NB> pf;
#pragma unroll
            for (int b = 0; b < NB; b++) {
              pf.rrs[b] = S.px_rrs[b][L];
              pf.pw[b] = S.px_pw[b][L];
            }
            pf.mean = S.px_mean[L];
            pf.r490 = pf.r550 = pf.r640 = 0.0;
            double xq[kN];
#pragma unroll
            for (int i = 0; i < kN; i++) xq[i] = S.rq_x[i][L];
            const double y = cost_f64<false, NB>(fp, args.sc, pf, xq, nullptr);
            S.rq_y[L] = y;
            __threadfence_block();
            *((volatile int32_t *)&S.rq_state[L]) = 2;
          }
          __syncwarp();
          __threadfence_block();
          if (lane == 0) atomicExch(&S.lock, 0);
        }
      }
    }
  }
  // exact-evaluation count for the roofline, and how the decisions went
  if (args.guard_stats) {
    atomicAdd(&S.stats[0], tally.exact);
    atomicAdd(&S.stats[1], tally.screened);
    atomicAdd(&S.stats[2], tally.deferred);
    atomicAdd(&S.stats[3], wait_trips);
    atomicAdd(&S.stats[4], busy_trips);
  }
  __syncthreads();
  if (tid == 0 && args.counters) atomicAdd(args.counters, S.served);
  if (tid == 0 && args.guard_stats)
    for (int i = 0; i < 5; i++) atomicAdd(args.guard_stats + i, S.stats[i]);
}

template <int NB, int BS>
cudaError_t launch_g(const InvertArgs &a, int grid, cudaStream_t s, int *occ) {
  const size_t smem = sizeof(Shared<NB, BS>);
  auto k = guarded_kernel<NB, BS>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  if (occ) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k, BS, smem);
  k<<<grid, BS, smem, s>>>(a);
  return cudaGetLastError();
}

template <int NB>
cudaError_t launch_gb(const InvertArgs &a, int block, int grid, cudaStream_t s, int *occ) {
  if (block == 256) return launch_g<NB, 256>(a, grid, s, occ);
  return launch_g<NB, 128>(a, grid, s, occ);
}

}  // namespace

cudaError_t launch_guarded(const InvertArgs &a, int block, int grid, cudaStream_t s) {
  if (a.fp.n_bands == 4) return launch_gb<4>(a, block, grid, s, nullptr);
  return launch_gb<8>(a, block, grid, s, nullptr);
}

int guarded_blocks_per_sm(const InvertArgs &a, int block) {
  int n = 0;
  cudaError_t e = a.fp.n_bands == 4 ? launch_gb<4>(a, block, 0, 0, &n)
                                    : launch_gb<8>(a, block, 0, 0, &n);
  return e == cudaSuccess ? n : 0;
}

}  // namespace photic
