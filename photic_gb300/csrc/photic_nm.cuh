// photic_nm.cuh -- resumable Nelder-Mead for one lane.
//
// The reference's nelmin (model/asa047.c:10-502) is a sequence of loops
// around calls of the cost function.  On the GPU each lane runs its own
// pixel, and lanes must reach the cost evaluation together to keep the
// warp converged where the work is.  So the method is restated as a state
// machine: step() consumes the cost of the point it last asked for and
// runs the bookkeeping up to the next point it needs, which it leaves in
// x[].  The sequence of points, comparisons and counters is the
// reference's; only the control flow is turned inside out.
//
// Vertices and vertex costs live in shared memory ([slot][thread], so a
// warp's accesses are conflict-free); vectors indexed only with
// compile-time indices live in registers.  The arithmetic type comes from
// the precision policy P (PrecF64: IEEE double in the reference's order;
// PrecDF: double-float on the FP32 pipes).
#pragma once
#include <stdint.h>

namespace photic {

enum NmPhase : int32_t {
  PH_INIT_BASE = 0,   // start point (vertex n)
  PH_INIT_VERT,       // vertex j of the initial simplex
  PH_REFLECT,
  PH_EXPAND,
  PH_CONTRACT_IN,     // contraction towards the worst vertex (l == 0)
  PH_CONTRACT_OUT,    // contraction towards the reflection (l == 1)
  PH_SHRINK,          // vertex j of a shrunk simplex
  PH_PROBE_PLUS,      // local-minimum probe xmin[i] + del
  PH_PROBE_MINUS,     // local-minimum probe xmin[i] - del
  PH_FINAL,           // re-evaluation at the kept optimum
};

// The kind of the pending simplex point of an iteration.
enum NmPoint : int32_t { PK_NONE = 0, PK_REFL, PK_EXPAND, PK_CONTRACT_IN, PK_CONTRACT_OUT };

// Loops over the simplex: fully unrolled for the single-scene simplex
// (n <= 8), so that the lane's vectors stay in registers, and rolled for the
// temporal fit (n up to 33).  (An unroll count that depends on a template
// parameter was not honoured: the n = 6 loops stayed rolled, and their
// dynamic indexes put the lane's vectors in local memory.)
template <int B, int E, bool kUnroll, class F>
__device__ __forceinline__ void nm_for(F &&f) {
  if constexpr (kUnroll) {
#pragma unroll
    for (int i = B; i < E; i++) f(i);
  } else {
#pragma unroll 1
    for (int i = B; i < E; i++) f(i);
  }
}

template <int N, class P, int BS>
struct NmLane {
  using T = typename P::T;
  static constexpr bool kU = N <= 8;  // unroll the loops over the simplex
  T *v, *f;  // shared: v[(j * N + i) * BS + tid], f[j * BS + tid]
  T x[N];    // point to evaluate next
  T cen[N], refl[N], trial[N], xmin[N], start[N], step[N];
  T ylo, fr, scale, var_limit;
  long long floor_lo;
  int32_t phase, jj, hi, lo, icount, numres, ifault, countdown, pk;
  int32_t kcount, konvge;

  __device__ __forceinline__ T &V(int j, int i) { return v[(j * N + i) * BS]; }
  __device__ __forceinline__ T &F(int j) { return f[j * BS]; }

  static __device__ __forceinline__ T pick(const T (&a)[N], int k) {
    T r = a[0];
    nm_for<1, N, kU>([&](int i) { if (i == k) r = a[i]; });
    return r;
  }
  static __device__ __forceinline__ void put(T (&a)[N], int k, T val) {
    nm_for<0, N, kU>([&](int i) { if (i == k) a[i] = val; });
  }

  // Begin a nelmin call from start[]/step[] (model/asa047.c:161-170).
  __device__ __forceinline__ void begin(T var_limit_, int32_t konvge_, int32_t kcount_) {
    konvge = konvge_;
    kcount = kcount_;
    countdown = konvge_;
    icount = 0;
    numres = 0;
    ifault = 0;
    scale = P::one();
    var_limit = var_limit_;
    restart_simplex();
  }

  __device__ __forceinline__ void restart_simplex() {
    nm_for<0, N, kU>([&](int i) {
      x[i] = start[i];
      V(N, i) = start[i];
    });
    phase = PH_INIT_BASE;
  }

  // Vertex j: the start point moved by step[j] * scale along coordinate j
  // (model/asa047.c:181-194).
  __device__ __forceinline__ void make_vertex(int j) {
    // one moved coordinate: computed once and placed, not once per slot
    const T sj = P::add(pick(start, j), P::mul(pick(step, j), scale));
    nm_for<0, N, kU>([&](int i) {
      const T s = i == j ? sj : start[i];
      x[i] = s;
      V(j, i) = s;
    });
    jj = j;
    phase = PH_INIT_VERT;
  }

  __device__ __forceinline__ void find_lo() {
    ylo = F(0);
    lo = 0;
    nm_for<1, N + 1, kU>([&](int j) {
      T fj = F(j);
      if (P::lt(fj, ylo)) {
        ylo = fj;
        lo = j;
      }
    });
  }

  // Top of the inner loop (model/asa047.c:213-250): budget check, worst
  // vertex, centroid of the others; the reflection is left pending (pk).
  // false: the loop ends.
  __device__ __forceinline__ bool inner_top() {
    if (kcount <= icount) return false;
    T yhi = F(0);
    hi = 0;
    nm_for<1, N + 1, kU>([&](int j) {
      T fj = F(j);
      if (P::lt(yhi, fj)) {
        yhi = fj;
        hi = j;
      }
    });
    nm_for<0, N, kU>([&](int i) {
      T z = P::zero();
      nm_for<0, N + 1, kU>([&](int j) { z = P::add(z, V(j, i)); });
      z = P::sub(z, V(hi, i));
      cen[i] = P::div_n(z, N);
    });
    pk = PK_REFL;
    phase = PH_REFLECT;
    return true;
  }

  // The pending point of the iteration, cen + c (a - b) with
  //   reflection          a = cen,   b = worst, c = 1   (model/asa047.c:251)
  //   expansion           a = refl,  b = cen,   c = 2   (:262)
  //   contraction inside  a = worst, b = cen,   c = 1/2 (:318)
  //   contraction outside a = refl,  b = cen,   c = 1/2 (:369)
  // c is a power of two, so the product is exact and each point equals the
  // reference's coordinate by coordinate (rcoeff = 1 multiplies exactly).
  // Written once for every kind, the lanes of a warp that need a point this
  // trip compute it together, whichever kind it is.
  __device__ __forceinline__ void make_point() {
    const bool r = pk == PK_REFL;
    const float c = pk == PK_EXPAND ? 2.0f : (r ? 1.0f : 0.5f);
    nm_for<0, N, kU>([&](int i) {
      const T w = V(hi, i);
      const T a = r ? cen[i] : (pk == PK_CONTRACT_IN ? w : refl[i]);
      const T b = r ? w : cen[i];
      const T p = P::add(cen[i], P::scale2(P::sub(a, b), c));
      x[i] = p;
      if (r) refl[i] = p;
      else trial[i] = p;
    });
  }

  __device__ __forceinline__ void replace_hi(const T (&p)[N], T y) {
    nm_for<0, N, kU>([&](int i) { V(hi, i) = p[i]; });
    F(hi) = y;
  }

  // End of an iteration (model/asa047.c:395-434).  true: the variance test
  // ends the inner loop.
  __device__ __forceinline__ bool iteration_end() {
    T fh = F(hi);
    if (P::lt(fh, ylo)) {
      ylo = fh;
      lo = hi;
    }
    countdown--;
    if (countdown > 0) return false;
    if (icount <= kcount) {
      countdown = konvge;
      T z = P::zero();
      nm_for<0, N + 1, kU>([&](int j) { z = P::add(z, F(j)); });
      T mean = P::div_n(z, N + 1);
      z = P::zero();
      nm_for<0, N + 1, kU>([&](int j) {
        T d = P::sub(F(j), mean);
        z = P::add(z, P::mul(d, d));
      });
      if (P::le(z, var_limit)) return true;
    }
    return false;
  }

  // Consume the cost y of x[] and advance to the next point.  Returns true
  // when the nelmin call has returned (xmin, F(lo), icount, numres, ifault
  // hold its results); the caller then starts another call or finishes.
  //
  // The bookkeeping after the cost is a fixed sequence of stages, each
  // guarded by the lane's state, so that the lanes of a warp needing the
  // same stage in a trip (the centroid, the pending point) run it together
  // instead of along one path per phase.
  __device__ __forceinline__ bool step_machine(T y) {
    enum { CS_NONE = -1, CS_READY, CS_TOP, CS_ITER_END, CS_END_INNER, CS_PROBE_PLUS,
           CS_PROBE_END, CS_NM_DONE };
    int cs = CS_NONE;
    pk = PK_NONE;
    switch (phase) {
      case PH_INIT_BASE:
        F(N) = y;
        icount++;
        make_vertex(0);
        break;
      case PH_INIT_VERT:
        F(jj) = y;
        icount++;
        if (jj + 1 < N) make_vertex(jj + 1);
        else cs = CS_READY;
        break;
      case PH_REFLECT:
        fr = y;
        icount++;
        if (P::lt(fr, ylo)) {
          pk = PK_EXPAND;
          phase = PH_EXPAND;
        } else {
          int worse = 0;
          nm_for<0, N + 1, kU>([&](int j) { if (P::lt(fr, F(j))) worse++; });
          if (worse > 1) {
            replace_hi(refl, fr);
            cs = CS_ITER_END;
          } else if (worse == 0) {
            pk = PK_CONTRACT_IN;
            phase = PH_CONTRACT_IN;
          } else {
            pk = PK_CONTRACT_OUT;
            phase = PH_CONTRACT_OUT;
          }
        }
        break;
      case PH_EXPAND:
        icount++;
        if (P::lt(fr, y)) replace_hi(refl, fr);
        else replace_hi(trial, y);
        cs = CS_ITER_END;
        break;
      case PH_CONTRACT_IN:
        icount++;
        if (P::lt(F(hi), y)) {
          // shrink every vertex towards the best (model/asa047.c:331-351)
          nm_for<0, N, kU>([&](int i) {
            T s = P::half(P::add(V(0, i), V(lo, i)));
            V(0, i) = s;
            x[i] = s;
          });
          jj = 0;
          phase = PH_SHRINK;
        } else {
          replace_hi(trial, y);
          cs = CS_ITER_END;
        }
        break;
      case PH_SHRINK:
        F(jj) = y;
        icount++;
        if (jj < N) {
          const int j = jj + 1;
          nm_for<0, N, kU>([&](int i) {
            T s = P::half(P::add(V(j, i), V(lo, i)));
            V(j, i) = s;
            x[i] = s;
          });
          jj = j;
        } else {
          cs = CS_READY;
        }
        break;
      case PH_CONTRACT_OUT:
        icount++;
        if (P::le(y, fr)) replace_hi(trial, y);
        else replace_hi(refl, fr);
        cs = CS_ITER_END;
        break;
      case PH_PROBE_PLUS: {
        icount++;
        if (P::trunc10(y) < floor_lo) {
          ifault = 2;
          cs = CS_PROBE_END;
        } else {
          const T del = P::eps_step(pick(step, jj));
          put(xmin, jj, P::sub(P::sub(pick(xmin, jj), del), del));
          nm_for<0, N, kU>([&](int i) { x[i] = xmin[i]; });
          phase = PH_PROBE_MINUS;
        }
        break;
      }
      case PH_PROBE_MINUS: {
        icount++;
        if (P::trunc10(y) < floor_lo) {
          ifault = 2;
          cs = CS_PROBE_END;
        } else {
          const T del = P::eps_step(pick(step, jj));
          put(xmin, jj, P::add(pick(xmin, jj), del));
          jj++;
          cs = (jj < N) ? CS_PROBE_PLUS : CS_PROBE_END;
        }
        break;
      }
      default:
        break;
    }
    // The transitions between the stages below only go forward
    // (READY -> TOP, ITER_END -> TOP | END_INNER, TOP -> END_INNER,
    // END_INNER -> PROBE_PLUS | NM_DONE), so one pass in this order
    // follows every chain the reference's loops can take.
    if (cs == CS_READY) {
      find_lo();
      cs = CS_TOP;
    }
    if (cs == CS_ITER_END) cs = iteration_end() ? CS_END_INNER : CS_TOP;
    if (cs == CS_TOP) cs = inner_top() ? CS_NONE : CS_END_INNER;
    if (cs == CS_END_INNER) {
      nm_for<0, N, kU>([&](int i) { xmin[i] = V(lo, i); });
      floor_lo = P::trunc10(F(lo));
      if (kcount < icount) {
        ifault = 2;
        cs = CS_NM_DONE;
      } else {
        ifault = 0;
        jj = 0;
        cs = CS_PROBE_PLUS;
      }
    }
    if (cs == CS_PROBE_PLUS) {
      const T del = P::eps_step(pick(step, jj));
      put(xmin, jj, P::add(pick(xmin, jj), del));
      nm_for<0, N, kU>([&](int i) { x[i] = xmin[i]; });
      phase = PH_PROBE_PLUS;
      cs = CS_NONE;
    }
    if (cs == CS_PROBE_END) {
      if (ifault == 0) {
        cs = CS_NM_DONE;
      } else {
        // restart from the probe point with a 1e-6 simplex
        nm_for<0, N, kU>([&](int i) { start[i] = xmin[i]; });
        scale = P::eps_scale();
        numres++;
        restart_simplex();
        cs = CS_NONE;
      }
    }
    if (pk != PK_NONE) make_point();
    return cs == CS_NM_DONE;
  }
};

}  // namespace photic
