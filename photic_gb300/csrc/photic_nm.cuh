// photic_nm.cuh -- resumable Nelder-Mead for one lane.
//
// The reference's nelmin (model/asa047.c:10-502) is a sequence of loops
// around calls of the cost function.  On the GPU each lane runs its own
// pixel, and lanes must reach the cost evaluation together to keep the
// warp converged where the work is.  So the method is restated as a state
// machine: advance() consumes the cost of the point it last asked for and
// runs the bookkeeping up to the next point it needs, which it leaves in
// x[].  The sequence of points, comparisons and counters is the
// reference's; only the control flow is turned inside out.
//
// Vertices and vertex costs live in shared memory ([slot][thread], so a
// warp's accesses are conflict-free); the vectors indexed with
// compile-time indices live in registers.
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
  PH_DONE
};

// Arithmetic hooks of the machine: T is the vertex/cost type.
template <class T>
struct NmOps;

template <>
struct NmOps<double> {
  static __device__ __forceinline__ double half() { return 0.5; }
  static __device__ __forceinline__ double two() { return 2.0; }
};

template <int N, class T, int BS>
struct NmLane {
  // shared-memory views: v[(j * N + i) * BS + tid], f[j * BS + tid]
  T *v, *f;
  // registers
  T x[N];                          // point to evaluate next
  T cen[N], refl[N], trial[N], xmin[N], start[N], step[N];
  T ylo, fr, scale;
  long long floor_lo;
  int32_t phase, jj, hi, lo, icount, numres, ifault, countdown;
  int32_t kcount, konvge;
  T var_limit;

  __device__ __forceinline__ T &V(int j, int i) { return v[(j * N + i) * BS]; }
  __device__ __forceinline__ T &F(int j) { return f[j * BS]; }

  template <class A>
  static __device__ __forceinline__ T pick(const A &a, int k) {
    T r = a[0];
#pragma unroll
    for (int i = 1; i < N; i++)
      if (i == k) r = a[i];
    return r;
  }
  template <class A>
  static __device__ __forceinline__ void put(A &a, int k, T val) {
#pragma unroll
    for (int i = 0; i < N; i++)
      if (i == k) a[i] = val;
  }

  // Begin a nelmin call from start[]/step[] (model/asa047.c:161-170).
  __device__ __forceinline__ void begin(T reqmin, int32_t konvge_, int32_t kcount_) {
    konvge = konvge_;
    kcount = kcount_;
    countdown = konvge_;
    icount = 0;
    numres = 0;
    ifault = 0;
    scale = T(1.0);
    var_limit = reqmin * T((double)N);
    restart_simplex();
  }

  __device__ __forceinline__ void restart_simplex() {
#pragma unroll
    for (int i = 0; i < N; i++) {
      x[i] = start[i];
      V(N, i) = start[i];
    }
    phase = PH_INIT_BASE;
  }

  // Vertex j: the start point moved by step[j] * scale along coordinate j
  // (model/asa047.c:181-194).
  __device__ __forceinline__ void make_vertex(int j) {
#pragma unroll
    for (int i = 0; i < N; i++) {
      T s = start[i];
      if (i == j) s = start[i] + step[i] * scale;
      x[i] = s;
      V(j, i) = s;
    }
    jj = j;
    phase = PH_INIT_VERT;
  }

  __device__ __forceinline__ void find_lo() {
    ylo = F(0);
    lo = 0;
#pragma unroll
    for (int j = 1; j <= N; j++) {
      T fj = F(j);
      if (fj < ylo) {
        ylo = fj;
        lo = j;
      }
    }
  }

  // Top of the inner loop (model/asa047.c:213-250): budget check, worst
  // vertex, centroid of the others, reflection.  Returns false when the
  // inner loop ends instead.
  __device__ __forceinline__ bool inner_top() {
    if (kcount <= icount) return false;
    T yhi = F(0);
    hi = 0;
#pragma unroll
    for (int j = 1; j <= N; j++) {
      T fj = F(j);
      if (yhi < fj) {
        yhi = fj;
        hi = j;
      }
    }
#pragma unroll
    for (int i = 0; i < N; i++) {
      T z = T(0.0);
#pragma unroll
      for (int j = 0; j <= N; j++) z = z + V(j, i);
      z = z - V(hi, i);
      cen[i] = z / T((double)N);
    }
#pragma unroll
    for (int i = 0; i < N; i++) {
      refl[i] = cen[i] + (cen[i] - V(hi, i));
      x[i] = refl[i];
    }
    phase = PH_REFLECT;
    return true;
  }

  __device__ __forceinline__ void replace_hi(const T *p, T y) {
#pragma unroll
    for (int i = 0; i < N; i++) V(hi, i) = p[i];
    F(hi) = y;
  }

  // End of an iteration (model/asa047.c:395-434).  Returns true when the
  // variance test ends the inner loop.
  __device__ __forceinline__ bool iteration_end() {
    T fh = F(hi);
    if (fh < ylo) {
      ylo = fh;
      lo = hi;
    }
    countdown--;
    if (countdown > 0) return false;
    if (icount <= kcount) {
      countdown = konvge;
      T z = T(0.0);
#pragma unroll
      for (int j = 0; j <= N; j++) z = z + F(j);
      T mean = z / T((double)(N + 1));
      z = T(0.0);
#pragma unroll
      for (int j = 0; j <= N; j++) {
        T d = F(j) - mean;
        z = z + d * d;
      }
      if (z <= var_limit) return true;
    }
    return false;
  }
};

}  // namespace photic
