// photic_invert.cu -- persistent, work-queue batched inversion of
// single-scene pixels (the plain method).
//
// One lane owns one pixel at a time and runs the whole per-pixel driver of
// samodel_optimise (model/samodel.c:1768-2115) with its 8 cold depth starts
// and early exit (model/samodel.c:2243-2407) on a resumable Nelder-Mead
// (photic_nm.cuh).  Every loop trip all lanes that hold a pixel evaluate
// the cost together; when a lane's pixel is finished it takes the next one
// from its warp's chunk, and a warp whose chunk is used up claims the next
// 32 pixels with one atomic and stages their spectra through shared memory
// with coalesced (float4 when the layout allows) loads.  Ragged iteration
// counts (a few hundred to several thousand evaluations per pixel) thus
// never leave a lane idle while work remains.
//
// Scratch: one 64-bit queue head and one 32-bit error word, supplied by
// the caller (photic_host.cpp allocates them stream-ordered).
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_fp64.cuh"
#include "photic_kernels.h"
#include "photic_nm.cuh"

namespace photic {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kN = 6;  // H, 100B, q, 100P, 100G, 100X

// Reference mask test (model/samodel.c:937-941): float tolerance compare
// with the nodata value, or negative reflectance.
__device__ __forceinline__ bool band_masked(float r, float nodata) {
  float diff = __fsub_rn(r, nodata);
  double big = fabs((double)r) < fabs((double)nodata) ? fabs((double)nodata) : fabs((double)r);
  return fabs((double)diff) <= big * (double)1.0e-6f || r < 0.0f;
}

struct Outputs {
  photic_outputs o;
  __device__ __forceinline__ void write_masked(int64_t p) const {
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
};

// Per-lane driver state around the Nelder-Mead machine.
struct Driver {
  int64_t pixel;
  int32_t start_k, n_starts, total, kept_evals, kept_start, kept_res, kept_fault, guard;
  double lowest;
  bool seeded;
};

template <int NB, int BS>
__global__ void __launch_bounds__(BS) invert_f64_kernel(InvertArgs args) {
  const FitParams &fp = args.fp;
  const SceneConsts &sc = args.sc;
  extern __shared__ unsigned char smem_raw[];
  double *sv = reinterpret_cast<double *>(smem_raw);           // [(N+1)*N][BS]
  double *sf = sv + (kN + 1) * kN * BS;                          // [N+1][BS]
  double *sbest = sf + (kN + 1) * BS;                            // [N][BS]
  float *schunk = reinterpret_cast<float *>(sbest + kN * BS);    // [BS/32][32][NB]

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  float *wchunk = schunk + warp * 32 * NB;
  const unsigned lt_mask = (1u << lane) - 1u;

  NmLane<kN, double, BS> m;
  m.v = sv + tid;
  m.f = sf + tid;
  double *best = sbest + tid;
  PixelF64<NB> px;
  Driver dr;
  dr.pixel = -1;
  Outputs out{args.out};

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
        int64_t p = chunk_base + lane;
        if (p < args.npix) {
          if (NB == 4 && args.vec4) {
            float4 v4 = __ldg(reinterpret_cast<const float4 *>(args.rrs) + p);
            wchunk[lane * NB + 0] = v4.x;
            wchunk[lane * NB + 1] = v4.y;
            wchunk[lane * NB + 2] = v4.z;
            wchunk[lane * NB + 3] = v4.w;
          } else {
#pragma unroll
            for (int b = 0; b < NB; b++)
              if (b < fp.n_bands)
                wchunk[lane * NB + b] = __ldg(args.rrs + p * args.pixel_stride + b * args.band_stride);
          }
        }
        __syncwarp();
      }
      const int rank = __popc(need & lt_mask);
      const int avail = (int)(chunk_end - chunk_next);
      const bool mine = ((need >> lane) & 1u) && rank < avail;
      const unsigned taken = __ballot_sync(kFull, mine);
      bool masked = false;
      if (mine) {
        const int64_t p = chunk_next + rank;
        float r[NB];
#pragma unroll
        for (int b = 0; b < NB; b++) r[b] = wchunk[(p - chunk_base) * NB + b];
#pragma unroll
        for (int b = 0; b < NB; b++)
          if (b < fp.n_bands && band_masked(r[b], fp.nodata)) masked = true;
        if (masked) {
          out.write_masked(p);
        } else {
          double rd[NB];
#pragma unroll
          for (int b = 0; b < NB; b++) rd[b] = (double)r[b];
          pixel_setup_f64<NB>(fp, sc, rd, px);
          dr.pixel = p;
          dr.total = 0;
          dr.kept_evals = 0;
          dr.kept_start = 0;
          dr.kept_res = 0;
          dr.kept_fault = 0;
          dr.guard = 0;
          dr.lowest = 1.0e4;
          dr.start_k = 0;
          dr.seeded = false;
#pragma unroll
          for (int i = 0; i < kN; i++) best[i * BS] = 0.0;
          if (args.seeds != nullptr) {
            const double *sd = args.seeds + p * kN;
            if (!isnan(sd[0])) {
              const double rel[kN] = {1.25, 1.5, 0.5, 2.0, 2.0, 2.0};
              dr.seeded = true;
#pragma unroll
              for (int i = 0; i < kN; i++) {
                m.start[i] = sd[i];
                m.step[i] = rel[i] * m.start[i];
              }
            }
          }
          dr.n_starts = dr.seeded ? 1 : fp.n_hstarts;
          if (!dr.seeded) {
            cold_start_f64<NB>(fp, px, m.start, m.step);
            m.start[0] = fp.hstarts[0];
            m.step[0] = 1.25 * m.start[0];
          }
          m.begin(fp.reqmin, fp.konvge, fp.kcount);
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
      if (m.phase == PH_FINAL) {
        CostDetailsF64 det;
        cost_f64<true, NB>(fp, sc, px, m.x, &det);
        const int64_t p = dr.pixel;
        const double H = fabs(m.x[0]);
        if (out.o.depth) out.o.depth[p] = (float)H;
        if (out.o.depth_f64) out.o.depth_f64[p] = H;
        if (out.o.P) out.o.P[p] = (float)(0.01 * fabs(m.x[3]));
        if (out.o.G) out.o.G[p] = (float)(0.01 * fabs(m.x[4]));
        if (out.o.X) out.o.X[p] = (float)(0.01 * fabs(m.x[5]));
        if (out.o.bottom_albedo) out.o.bottom_albedo[p] = (float)det.bottom_albedo;
        if (out.o.model_error) out.o.model_error[p] = (float)det.model_error;
        if (out.o.rrs_error) out.o.rrs_error[p] = (float)det.rrs_error;
        if (out.o.K_min) out.o.K_min[p] = (float)det.K_min;
        if (out.o.iod) out.o.iod[p] = (float)det.iod;
        if (out.o.evals) out.o.evals[p] = dr.total;
        if (out.o.evals_kept) out.o.evals_kept[p] = dr.kept_evals;
        if (out.o.status)
          out.o.status[p] = PHOTIC_PX_FITTED | (dr.kept_fault == 0 ? PHOTIC_PX_CONVERGED : 0) |
                            (dr.kept_start << 16);
        has = false;
      } else {
        const double y = cost_f64<false, NB>(fp, sc, px, m.x, nullptr);
        if (++dr.guard > guard_cap) {
          // Defensive cap on evaluations per pixel; the method itself is
          // bounded by kcount per start, so reaching this means a defect.
          atomicOr(args.error, PHOTIC_DEVERR_EVAL_CAP);
          if (out.o.status) out.o.status[dr.pixel] = PHOTIC_PX_INVALID;
          has = false;
        } else {
          // ---- advance the Nelder-Mead machine --------------------------
          int cs = -1;  // control state after consuming y
          enum { CS_READY, CS_TOP, CS_ITER_END, CS_END_INNER, CS_PROBE_PLUS, CS_PROBE_END,
                 CS_NM_DONE };
          switch (m.phase) {
            case PH_INIT_BASE:
              m.F(kN) = y;
              m.icount++;
              m.make_vertex(0);
              break;
            case PH_INIT_VERT:
              m.F(m.jj) = y;
              m.icount++;
              if (m.jj + 1 < kN) m.make_vertex(m.jj + 1);
              else cs = CS_READY;
              break;
            case PH_REFLECT:
              m.fr = y;
              m.icount++;
              if (m.fr < m.ylo) {
#pragma unroll
                for (int i = 0; i < kN; i++) {
                  m.trial[i] = m.cen[i] + 2.0 * (m.refl[i] - m.cen[i]);
                  m.x[i] = m.trial[i];
                }
                m.phase = PH_EXPAND;
              } else {
                int worse = 0;
#pragma unroll
                for (int j = 0; j <= kN; j++)
                  if (m.fr < m.F(j)) worse++;
                if (worse > 1) {
                  m.replace_hi(m.refl, m.fr);
                  cs = CS_ITER_END;
                } else if (worse == 0) {
#pragma unroll
                  for (int i = 0; i < kN; i++) {
                    m.trial[i] = m.cen[i] + 0.5 * (m.V(m.hi, i) - m.cen[i]);
                    m.x[i] = m.trial[i];
                  }
                  m.phase = PH_CONTRACT_IN;
                } else {
#pragma unroll
                  for (int i = 0; i < kN; i++) {
                    m.trial[i] = m.cen[i] + 0.5 * (m.refl[i] - m.cen[i]);
                    m.x[i] = m.trial[i];
                  }
                  m.phase = PH_CONTRACT_OUT;
                }
              }
              break;
            case PH_EXPAND:
              m.icount++;
              if (m.fr < y) m.replace_hi(m.refl, m.fr);
              else m.replace_hi(m.trial, y);
              cs = CS_ITER_END;
              break;
            case PH_CONTRACT_IN:
              m.icount++;
              if (m.F(m.hi) < y) {
                // shrink every vertex towards the best (model/asa047.c:331-351)
#pragma unroll
                for (int i = 0; i < kN; i++) {
                  double s = (m.V(0, i) + m.V(m.lo, i)) * 0.5;
                  m.V(0, i) = s;
                  m.x[i] = s;
                }
                m.jj = 0;
                m.phase = PH_SHRINK;
              } else {
                m.replace_hi(m.trial, y);
                cs = CS_ITER_END;
              }
              break;
            case PH_SHRINK:
              m.F(m.jj) = y;
              m.icount++;
              if (m.jj < kN) {
                const int j = m.jj + 1;
#pragma unroll
                for (int i = 0; i < kN; i++) {
                  double s = (m.V(j, i) + m.V(m.lo, i)) * 0.5;
                  m.V(j, i) = s;
                  m.x[i] = s;
                }
                m.jj = j;
              } else {
                cs = CS_READY;
              }
              break;
            case PH_CONTRACT_OUT:
              m.icount++;
              if (y <= m.fr) m.replace_hi(m.trial, y);
              else m.replace_hi(m.refl, m.fr);
              cs = CS_ITER_END;
              break;
            case PH_PROBE_PLUS: {
              m.icount++;
              if (trunc10(y) < m.floor_lo) {
                m.ifault = 2;
                cs = CS_PROBE_END;
              } else {
                const double del = NmLane<kN, double, BS>::pick(m.step, m.jj) * 1.0e-6;
                const double xi = NmLane<kN, double, BS>::pick(m.xmin, m.jj);
                NmLane<kN, double, BS>::put(m.xmin, m.jj, xi - del - del);
#pragma unroll
                for (int i = 0; i < kN; i++) m.x[i] = m.xmin[i];
                m.phase = PH_PROBE_MINUS;
              }
              break;
            }
            case PH_PROBE_MINUS: {
              m.icount++;
              if (trunc10(y) < m.floor_lo) {
                m.ifault = 2;
                cs = CS_PROBE_END;
              } else {
                const double del = NmLane<kN, double, BS>::pick(m.step, m.jj) * 1.0e-6;
                const double xi = NmLane<kN, double, BS>::pick(m.xmin, m.jj);
                NmLane<kN, double, BS>::put(m.xmin, m.jj, xi + del);
                m.jj++;
                cs = (m.jj < kN) ? CS_PROBE_PLUS : CS_PROBE_END;
              }
              break;
            }
            default:
              break;
          }
          // Run the bookkeeping until the next point to evaluate.
          while (cs >= 0) {
            switch (cs) {
              case CS_READY:
                m.find_lo();
                cs = CS_TOP;
                break;
              case CS_TOP:
                cs = m.inner_top() ? -1 : CS_END_INNER;
                break;
              case CS_ITER_END:
                cs = m.iteration_end() ? CS_END_INNER : CS_TOP;
                break;
              case CS_END_INNER: {
#pragma unroll
                for (int i = 0; i < kN; i++) m.xmin[i] = m.V(m.lo, i);
                m.floor_lo = trunc10(m.F(m.lo));
                if (m.kcount < m.icount) {
                  m.ifault = 2;
                  cs = CS_NM_DONE;
                } else {
                  m.ifault = 0;
                  m.jj = 0;
                  cs = CS_PROBE_PLUS;
                }
                break;
              }
              case CS_PROBE_PLUS: {
                const double del = NmLane<kN, double, BS>::pick(m.step, m.jj) * 1.0e-6;
                const double xi = NmLane<kN, double, BS>::pick(m.xmin, m.jj);
                NmLane<kN, double, BS>::put(m.xmin, m.jj, xi + del);
#pragma unroll
                for (int i = 0; i < kN; i++) m.x[i] = m.xmin[i];
                m.phase = PH_PROBE_PLUS;
                cs = -1;
                break;
              }
              case CS_PROBE_END:
                if (m.ifault == 0) {
                  cs = CS_NM_DONE;
                } else {
                  // restart from the probe point with a 1e-6 simplex
#pragma unroll
                  for (int i = 0; i < kN; i++) m.start[i] = m.xmin[i];
                  m.scale = 1.0e-6;
                  m.numres++;
                  m.restart_simplex();
                  cs = -1;
                }
                break;
              case CS_NM_DONE: {
                // nelmin returned: ynewlo = F(lo), xmin, icount, numres, ifault
                const double ynewlo = m.F(m.lo);
                dr.total += m.icount;
                bool finish = false;
                if (ynewlo < dr.lowest) {
                  dr.lowest = ynewlo;
#pragma unroll
                  for (int i = 0; i < kN; i++) best[i * BS] = m.xmin[i];
                  dr.kept_evals = m.icount;
                  dr.kept_res = m.numres;
                  dr.kept_start = dr.start_k;
                  dr.kept_fault = m.ifault;
                  if (dr.lowest < args.early_exit) finish = true;
                }
                dr.start_k++;
                if (!finish && dr.start_k < dr.n_starts) {
                  double h = fp.hstarts[0];
                  for (int k = 1; k < kMaxHStarts; k++)
                    if (k == dr.start_k) h = fp.hstarts[k];
                  cold_start_f64<NB>(fp, px, m.start, m.step);
                  m.start[0] = h;
                  m.step[0] = 1.25 * m.start[0];
                  m.begin(fp.reqmin, fp.konvge, fp.kcount);
                } else {
#pragma unroll
                  for (int i = 0; i < kN; i++) m.x[i] = best[i * BS];
                  m.phase = PH_FINAL;
                }
                cs = -1;
                break;
              }
              default:
                cs = -1;
                break;
            }
          }
        }
      }
    }
  }
}

}  // namespace

template <int NB, int BS>
static int occupancy_nb() {
  size_t smem = smem_bytes_f64(BS, NB);
  auto k = invert_f64_kernel<NB, BS>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, BS, smem) != cudaSuccess) return 0;
  return n;
}

int invert_f64_blocks_per_sm(int nb, int block) {
  if (nb == 4) {
    if (block == 64) return occupancy_nb<4, 64>();
    if (block == 256) return occupancy_nb<4, 256>();
    return occupancy_nb<4, 128>();
  }
  if (block == 64) return occupancy_nb<8, 64>();
  if (block == 256) return occupancy_nb<8, 256>();
  return occupancy_nb<8, 128>();
}

template <int NB>
static cudaError_t launch_nb(const InvertArgs &a, int block, int grid, cudaStream_t s) {
  if (block == 128) {
    size_t smem = smem_bytes_f64(128, NB);
    auto k = invert_f64_kernel<NB, 128>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, 128, smem, s>>>(a);
  } else if (block == 64) {
    size_t smem = smem_bytes_f64(64, NB);
    auto k = invert_f64_kernel<NB, 64>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, 64, smem, s>>>(a);
  } else {
    size_t smem = smem_bytes_f64(256, NB);
    auto k = invert_f64_kernel<NB, 256>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k<<<grid, 256, smem, s>>>(a);
  }
  return cudaGetLastError();
}

size_t smem_bytes_f64(int block, int nb) {
  return (size_t)block * sizeof(double) * ((kN + 1) * kN + (kN + 1) + kN) +
         (size_t)(block / 32) * 32 * nb * sizeof(float);
}

cudaError_t launch_invert_f64(const InvertArgs &a, int block, int grid, cudaStream_t s) {
  if (a.fp.n_bands == 4) return launch_nb<4>(a, block, grid, s);
  return launch_nb<8>(a, block, grid, s);
}

}  // namespace photic
