// photic_nmgroup.cuh -- Nelder-Mead (model/asa047.c:10-502) for a group of
// G lanes sharing one pixel: the resumable state machine of photic_nm.cuh
// with the coordinate loops cut to each lane's own coordinates.  Lane l owns
// coordinate l (and l + G, ... up to C slots) of every vertex, the centroid
// and the trial points; the vertex costs and every decision taken on them
// are replicated in all lanes of the group, each lane keeping its own copy
// of the costs -- or, with kSharedF (a group of a whole warp), one copy
// that every write reaches between two warp barriers.  The simplex size is a
// template constant (NT > 0) or set at run time (NT = 0, member nrt), for
// pixels whose parameter count varies.
#pragma once
#include <stdint.h>

#include "photic_fp64.cuh"
#include "photic_nm.cuh"

namespace photic {

// Group-distributed Nelder-Mead: the state machine of NmLane with the
// coordinate loops cut to the lane's own coordinates.
template <int NT, int C, int G, int CG, bool kSharedF = false>
struct NmGroup {
  int nrt;             // the simplex size when NT <= 0 (set before begin)
  double *V, *Fv, *X;  // shared: V[j * CG + i], this lane's costs Fv[j * G] (or the
                       // group's Fv[j] with kSharedF), X[i]
  int gl;              // lane within the group
  unsigned gmask;      // the group's lanes
  double cen[C], refl[C], trial[C], xmin[C], start[C], step[C];
  double ylo, fr, scale, var_limit;
  double inv_n, inv_n1;  // RN(1 / n), RN(1 / (n + 1)) for the centroid and the variance test
  long long floor_lo;
  int32_t phase, jj, hi, lo, icount, numres, ifault, countdown, kcount, konvge;

  __device__ __forceinline__ int dim() const { return NT > 0 ? NT : nrt; }
  __device__ __forceinline__ int coord(int t) const { return gl + t * G; }
  __device__ __forceinline__ bool own(int t) const { return coord(t) < dim(); }
  // The slot holding coordinate i on this lane, -1 if another lane owns it.
  // (Matching i against coord(t) slot by slot instead lost the match on
  // the second slot in the compiled kernel: the stepped vertex of the last
  // coordinate came out unstepped.)
  __device__ __forceinline__ int slot_of(int i) const { return (i % G) == gl ? i / G : -1; }
  __device__ __forceinline__ double &Vv(int j, int i) { return V[j * CG + i]; }
  __device__ __forceinline__ double &F(int j) { return Fv[kSharedF ? j : j * G]; }
  // A cost write.  With one copy for the warp, every lane has made the
  // step's reads before any lane writes, and sees the write after it:
  // the lanes take the same decisions, so they all reach both barriers.
  __device__ __forceinline__ void setF(int j, double y) {
    if constexpr (kSharedF) {
#if defined(__CUDA_ARCH__)
      __syncwarp(gmask);
#endif
      Fv[j] = y;
#if defined(__CUDA_ARCH__)
      __syncwarp(gmask);
#endif
    } else {
      Fv[j * G] = y;
    }
  }

  // Every slot gets a defined value, also those of coordinates the lane
  // does not own (they are computed on but never stored).
  __device__ __forceinline__ void clear() {
#pragma unroll
    for (int t = 0; t < C; t++) {
      cen[t] = 0.0;
      refl[t] = 0.0;
      trial[t] = 0.0;
      xmin[t] = 0.0;
      start[t] = 0.0;
      step[t] = 0.0;
    }
    ylo = fr = 0.0;
    inv_n = inv_n1 = 1.0;
    scale = 1.0;
    floor_lo = 0;
    phase = jj = hi = lo = icount = numres = ifault = countdown = 0;
  }

  __device__ __forceinline__ void begin(double var_limit_, int32_t konvge_, int32_t kcount_) {
    konvge = konvge_;
    kcount = kcount_;
    countdown = konvge_;
    icount = 0;
    numres = 0;
    ifault = 0;
    scale = 1.0;
    var_limit = var_limit_;
    inv_n = 1.0 / (double)dim();
    inv_n1 = 1.0 / (double)(dim() + 1);
    restart_simplex();
  }

  __device__ __forceinline__ void restart_simplex() {
#pragma unroll
    for (int t = 0; t < C; t++)
      if (own(t)) {
        X[coord(t)] = start[t];
        Vv(dim(), coord(t)) = start[t];
      }
    phase = PH_INIT_BASE;
  }

  __device__ __forceinline__ void make_vertex(int j) {
    const int ts = slot_of(j);
#pragma unroll
    for (int t = 0; t < C; t++)
      if (own(t)) {
        const int i = coord(t);
        double s = start[t];
        if (t == ts) s = start[t] + step[t] * scale;
        X[i] = s;
        Vv(j, i) = s;
      }
    jj = j;
    phase = PH_INIT_VERT;
  }

  __device__ __forceinline__ void find_lo() {
    ylo = F(0);
    lo = 0;
    for (int j = 1; j <= dim(); j++) {
      const double fj = F(j);
      if (fj < ylo) {
        ylo = fj;
        lo = j;
      }
    }
  }

  // The worst vertex: the first index of the largest cost, a NaN cost
  // never replacing the running one (a NaN at index 0 is kept, model/
  // asa047.c:221-231).  With one cost copy for the warp, each lane scans
  // the vertices j = lane, lane + 32, ... and the warp combines the lanes'
  // (cost, index) by the larger cost, the smaller index on a tie.
  __device__ __forceinline__ int worst_vertex() {
    if constexpr (kSharedF) {
#if defined(__CUDA_ARCH__)
      const double f0 = F(0);
      if (f0 != f0) return 0;
      double v = 0.0;
      int idx = 0x7fffffff;
      for (int j = gl; j <= dim(); j += G) {
        const double f = F(j);
        if (f == f && (idx == 0x7fffffff || v < f)) {
          v = f;
          idx = j;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(gmask, v, o);
        const int oi = __shfl_xor_sync(gmask, idx, o);
        if (oi != 0x7fffffff &&
            (idx == 0x7fffffff || v < ov || (!(ov < v) && oi < idx))) {
          v = ov;
          idx = oi;
        }
      }
      return idx;
#endif
    }
    double yhi = F(0);
    int h = 0;
    for (int j = 1; j <= dim(); j++) {
      const double fj = F(j);
      if (yhi < fj) {
        yhi = fj;
        h = j;
      }
    }
    return h;
  }

  // How many vertices cost more than fr (model/asa047.c:294-301): a count,
  // so with one cost copy the lanes count their vertices and the warp adds.
  __device__ __forceinline__ int count_worse(double fr_) {
    if constexpr (kSharedF) {
#if defined(__CUDA_ARCH__)
      int c = 0;
      for (int j = gl; j <= dim(); j += G)
        if (fr_ < F(j)) c++;
      return (int)__reduce_add_sync(gmask, (unsigned)c);
#endif
    }
    int worse = 0;
    for (int j = 0; j <= dim(); j++)
      if (fr_ < F(j)) worse++;
    return worse;
  }

  __device__ __forceinline__ bool inner_top() {
    if (kcount <= icount) return false;
    hi = worst_vertex();
#pragma unroll
    for (int t = 0; t < C; t++)
      if (own(t)) {
        const int i = coord(t);
        double z = 0.0;
        for (int j = 0; j <= dim(); j++) z = z + Vv(j, i);
        z = z - Vv(hi, i);
        cen[t] = fm::div_by(z, (double)dim(), inv_n);
        refl[t] = cen[t] + (cen[t] - Vv(hi, i));
        X[i] = refl[t];
      }
    phase = PH_REFLECT;
    return true;
  }

  // Each lane keeps its own copy of the vertex costs (the same values in
  // every lane of the group), so no lane ever reads a cost another lane is
  // writing, whatever the lanes' relative progress; or one shared copy
  // written between barriers (setF).
  __device__ __forceinline__ void replace_hi(const double (&p)[C], double y) {
#pragma unroll
    for (int t = 0; t < C; t++)
      if (own(t)) Vv(hi, coord(t)) = p[t];
    setF(hi, y);
  }

  __device__ __forceinline__ bool iteration_end() {
    const double fh = F(hi);
    if (fh < ylo) {
      ylo = fh;
      lo = hi;
    }
    countdown--;
    if (countdown > 0) return false;
    if (icount <= kcount) {
      countdown = konvge;
      double z = 0.0;
      for (int j = 0; j <= dim(); j++) z = z + F(j);
      const double mean = fm::div_by(z, (double)(dim() + 1), inv_n1);
      z = 0.0;
      for (int j = 0; j <= dim(); j++) {
        const double d = F(j) - mean;
        z = z + d * d;
      }
      if (z <= var_limit) return true;
    }
    return false;
  }

  __device__ __forceinline__ void set_x_from(const double (&p)[C]) {
#pragma unroll
    for (int t = 0; t < C; t++)
      if (own(t)) X[coord(t)] = p[t];
  }

  // xmin[jj] += sgn * del on the lane that owns coordinate jj.
  __device__ __forceinline__ void probe_move(int sgn_twice) {
    const int ts = slot_of(jj);
#pragma unroll
    for (int t = 0; t < C; t++)
      if (t == ts) {
        const double del = step[t] * 1.0e-6;
        if (sgn_twice > 0) xmin[t] = xmin[t] + del;
        else if (sgn_twice < 0) xmin[t] = (xmin[t] - del) - del;
        else xmin[t] = xmin[t] + del;  // back to the centre after the minus probe
      }
  }

  __device__ __forceinline__ bool step_machine(double y) {
    enum { CS_NONE = -1, CS_READY, CS_TOP, CS_ITER_END, CS_END_INNER, CS_PROBE_PLUS,
           CS_PROBE_END, CS_NM_DONE };
    int cs = CS_NONE;
    switch (phase) {
      case PH_INIT_BASE:
        setF(dim(), y);
        icount++;
        make_vertex(0);
        break;
      case PH_INIT_VERT:
        setF(jj, y);
        icount++;
        if (jj + 1 < dim()) make_vertex(jj + 1);
        else cs = CS_READY;
        break;
      case PH_REFLECT:
        fr = y;
        icount++;
        if (fr < ylo) {
#pragma unroll
          for (int t = 0; t < C; t++) trial[t] = cen[t] + 2.0 * (refl[t] - cen[t]);
          set_x_from(trial);
          phase = PH_EXPAND;
        } else {
          const int worse = count_worse(fr);
          if (worse > 1) {
            replace_hi(refl, fr);
            cs = CS_ITER_END;
          } else if (worse == 0) {
#pragma unroll
            for (int t = 0; t < C; t++)
              if (own(t)) trial[t] = cen[t] + (Vv(hi, coord(t)) - cen[t]) * 0.5;
            set_x_from(trial);
            phase = PH_CONTRACT_IN;
          } else {
#pragma unroll
            for (int t = 0; t < C; t++) trial[t] = cen[t] + (refl[t] - cen[t]) * 0.5;
            set_x_from(trial);
            phase = PH_CONTRACT_OUT;
          }
        }
        break;
      case PH_EXPAND:
        icount++;
        if (fr < y) replace_hi(refl, fr);
        else replace_hi(trial, y);
        cs = CS_ITER_END;
        break;
      case PH_CONTRACT_IN: {
        icount++;
        const bool shrink = F(hi) < y;
        if (shrink) {
#pragma unroll
          for (int t = 0; t < C; t++)
            if (own(t)) {
              const int i = coord(t);
              const double s = (Vv(0, i) + Vv(lo, i)) * 0.5;
              Vv(0, i) = s;
              X[i] = s;
            }
          jj = 0;
          phase = PH_SHRINK;
        } else {
          replace_hi(trial, y);
          cs = CS_ITER_END;
        }
        break;
      }
      case PH_SHRINK:
        setF(jj, y);
        icount++;
        if (jj < dim()) {
          const int j = jj + 1;
#pragma unroll
          for (int t = 0; t < C; t++)
            if (own(t)) {
              const int i = coord(t);
              const double s = (Vv(j, i) + Vv(lo, i)) * 0.5;
              Vv(j, i) = s;
              X[i] = s;
            }
          jj = j;
        } else {
          cs = CS_READY;
        }
        break;
      case PH_CONTRACT_OUT:
        icount++;
        if (y <= fr) replace_hi(trial, y);
        else replace_hi(refl, fr);
        cs = CS_ITER_END;
        break;
      case PH_PROBE_PLUS:
        icount++;
        if (trunc10(y) < floor_lo) {
          ifault = 2;
          cs = CS_PROBE_END;
        } else {
          probe_move(-1);
          set_x_from(xmin);
          phase = PH_PROBE_MINUS;
        }
        break;
      case PH_PROBE_MINUS:
        icount++;
        if (trunc10(y) < floor_lo) {
          ifault = 2;
          cs = CS_PROBE_END;
        } else {
          probe_move(0);
          jj++;
          cs = (jj < dim()) ? CS_PROBE_PLUS : CS_PROBE_END;
        }
        break;
      default:
        break;
    }
    while (cs != CS_NONE) {
      switch (cs) {
        case CS_READY:
          find_lo();
          cs = CS_TOP;
          break;
        case CS_TOP:
          cs = inner_top() ? CS_NONE : CS_END_INNER;
          break;
        case CS_ITER_END:
          cs = iteration_end() ? CS_END_INNER : CS_TOP;
          break;
        case CS_END_INNER:
#pragma unroll
          for (int t = 0; t < C; t++)
            if (own(t)) xmin[t] = Vv(lo, coord(t));
          floor_lo = trunc10(F(lo));
          if (kcount < icount) {
            ifault = 2;
            cs = CS_NM_DONE;
          } else {
            ifault = 0;
            jj = 0;
            cs = CS_PROBE_PLUS;
          }
          break;
        case CS_PROBE_PLUS:
          probe_move(+1);
          set_x_from(xmin);
          phase = PH_PROBE_PLUS;
          cs = CS_NONE;
          break;
        case CS_PROBE_END:
          if (ifault == 0) {
            cs = CS_NM_DONE;
          } else {
#pragma unroll
            for (int t = 0; t < C; t++) start[t] = xmin[t];
            scale = 1.0e-6;
            numres++;
            restart_simplex();
            cs = CS_NONE;
          }
          break;
        case CS_NM_DONE:
          return true;
        default:
          cs = CS_NONE;
          break;
      }
    }
    return false;
  }
};

}  // namespace photic
