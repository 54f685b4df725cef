// photic_gemm.cu -- BF16 "TN" GEMM on the tcgen05 tensor cores:
//   C[M x N] = A[M x K] * B[N x K]^T  (A, B row-major BF16, K contiguous)
// with the FP32 accumulator in tensor memory and a fused epilogue.  It is
// the building block of the surrogate MLP (photic_mlp.cu): forward layers
// (bias + SiLU), input gradients (times SiLU') and weight gradients.
//
// One CTA (4 warps) owns a 128 x BN output tile (or, split-K, one slice of
// K of it: the weight-gradient products have 128 x 128 outputs and K = the
// batch, so their K is spread over CTAs and the partial sums are added in a
// fixed order by a second kernel).  K is consumed in chunks
// of 64: all threads stage the A and B chunks into shared memory in the
// canonical no-swizzle core-matrix layout (16-byte vector loads), one
// thread issues four K=16 MMAs and commits them to an mbarrier, everyone
// waits (bounded), and the epilogue reads the accumulator back with
// tcgen05.ld, one TMEM lane (= output row) per thread.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "photic_kernels.h"
#include "photic_tc.cuh"

namespace photic {

namespace {

constexpr int kBM = 128, kBN = 128, kBK = 64;
constexpr uint32_t kTmemCols = 256;        // >= any N the descriptor can name here
constexpr uint32_t kWaitLimit = 1u << 26;  // bounded mbarrier spin

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// Stage rows [r0, r0+rows) x cols [k0, k0+64) of a row-major BF16 matrix
// into the core-matrix layout: element (r, k) at byte
// ((r/8)*8 + k/8)*128 + (r%8)*16 + (k%8)*2.  Out-of-range parts are zero.
__device__ __forceinline__ void stage(const __nv_bfloat16 *src, int ld, int nrows_total,
                                      int r0, int rows, int k0, int K, unsigned char *dst) {
  const int vecs = rows * (kBK / 8);
  for (int v = threadIdx.x; v < vecs; v += blockDim.x) {
    const int r = v >> 3, c = v & 7;
    const int gr = r0 + r, gk = k0 + c * 8;
    uint4 val = make_uint4(0u, 0u, 0u, 0u);
    if (gr < nrows_total && gk < K)
      val = *reinterpret_cast<const uint4 *>(src + (size_t)gr * ld + gk);
    *reinterpret_cast<uint4 *>(dst + (((r >> 3) * 8 + c) * 128 + (r & 7) * 16)) = val;
  }
}

__global__ void __launch_bounds__(128) tn_gemm_kernel(const __grid_constant__ GemmArgs g) {
  const __nv_bfloat16 *gA = reinterpret_cast<const __nv_bfloat16 *>(g.A);
  const __nv_bfloat16 *gB = reinterpret_cast<const __nv_bfloat16 *>(g.B);
  __nv_bfloat16 *gO = reinterpret_cast<__nv_bfloat16 *>(g.O);
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char *sA = smem;                      // kBM x kBK
  unsigned char *sB = smem + kBM * kBK * 2;      // kBN x kBK
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;

  const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
  const int ncols = min(kBN, g.N - n0);          // valid output columns of this tile
  const int mma_n = (ncols + 15) / 16 * 16;      // MMA N: multiple of 16, <= 128
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) tc::tmem_alloc(&tmem_slot, kTmemCols);
  if (threadIdx.x == 0) tc::mbar_init(&mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = tc::make_idesc_bf16(kBM, mma_n);

  bool ok = true;
  // split-K: CTA z takes chunks [c0, c1) of K and writes a partial sum
  const int nchunks = (g.K + kBK - 1) / kBK;
  const int per = g.ksplit > 1 ? (nchunks + g.ksplit - 1) / g.ksplit : nchunks;
  const int c0 = (int)blockIdx.z * per;
  const int c1 = min(nchunks, c0 + per);
  for (int kc = c0; kc < c1 && ok; kc++) {
    const int k0 = kc * kBK;
    stage(gA, g.lda, g.M, m0, kBM, k0, g.K, sA);
    stage(gB, g.ldb, g.N, n0, kBN, k0, g.K, sB);
    tc::fence_smem_async();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc::fence_after_sync();
      const uint32_t a0 = tc::smem_u32(sA), b0 = tc::smem_u32(sB);
#pragma unroll
      for (int kk = 0; kk < kBK / 16; kk++) {
        if (k0 + kk * 16 < g.K) {
          const uint64_t ad = tc::make_desc(a0 + kk * 256, g.lbo, g.sbo);
          const uint64_t bd = tc::make_desc(b0 + kk * 256, g.lbo, g.sbo);
          tc::mma_bf16(tmem, ad, bd, idesc, (kc > c0 || kk > 0) ? 1u : 0u);
        }
      }
      tc::mma_commit(&mbar);
    }
    if (!tc::mbar_wait(&mbar, (uint32_t)((kc - c0) & 1), kWaitLimit)) {
      ok = false;
      if (threadIdx.x == 0) atomicOr(g.error, PHOTIC_DEVERR_MMA_TIMEOUT);
      // give the tensor core a second bounded chance to finish before the
      // shared memory and TMEM go away
      tc::mbar_wait(&mbar, (uint32_t)((kc - c0) & 1), kWaitLimit);
    }
    tc::fence_after_sync();
    __syncthreads();
  }

  if (ok && c1 <= c0) {
    // an empty split contributes zeros
    const int row = m0 + warp * 32 + lane;
    if (row < g.M)
      for (int j = 0; j < ncols; j++)
        g.partial[((size_t)blockIdx.z * g.M + row) * g.N + n0 + j] = 0.0f;
  } else if (ok) {
    const int row = m0 + warp * 32 + lane;
    for (int cc = 0; cc < mma_n; cc += 16) {
      float v[16];
      tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)cc, v);
      if (row < g.M) {
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int col = n0 + cc + j;
          if (cc + j >= ncols) break;
          float acc = v[j];
          if (g.partial) {
            g.partial[((size_t)blockIdx.z * g.M + row) * g.N + col] = acc;
            continue;
          }
          switch (g.epi) {
            case EPI_F32:
              g.C[(size_t)row * g.ldc + col] = acc;
              break;
            case EPI_BIAS_F32:
              g.C[(size_t)row * g.ldc + col] = acc + g.bias[col];
              break;
            case EPI_BIAS_SILU: {
              const float z = acc + g.bias[col];
              if (g.Z) g.Z[(size_t)row * g.ldz + col] = z;
              gO[(size_t)row * g.ldo + col] = __float2bfloat16(silu(z));
              break;
            }
            case EPI_DSILU: {
              const float z = g.Z[(size_t)row * g.ldz + col];
              gO[(size_t)row * g.ldo + col] = __float2bfloat16(acc * dsilu(z));
              break;
            }
            default:
              break;
          }
        }
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_free(tmem, kTmemCols);
}

// C = sum over splits of the partial products, in split order (the sum is
// the same on every run).
__global__ void splitk_reduce_kernel(const float *partial, int S, int M, int N, float *C,
                                     int ldc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)M * N) return;
  const int r = (int)(i / N), c = (int)(i % N);
  float s = 0.0f;
  for (int z = 0; z < S; z++) s += partial[(size_t)z * M * N + i];
  C[(size_t)r * ldc + c] = s;
}

}  // namespace

// Dynamic shared memory is sized to keep at most two CTAs per SM, so the
// TMEM of resident CTAs (2 x 256 of 512 columns) never over-subscribes.
size_t gemm_smem_bytes() { return 96 * 1024; }

cudaError_t launch_gemm(const GemmArgs &g, cudaStream_t s) {
  if (g.M <= 0 || g.N <= 0) return cudaSuccess;
  const size_t smem = gemm_smem_bytes();
  cudaError_t e = cudaFuncSetAttribute(tn_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  const int nchunks = (g.K + kBK - 1) / kBK;
  GemmArgs a = g;
  int S = 1;
  if (g.ksplit > 1 && g.partial && g.epi == EPI_F32 && nchunks > 1) {
    const int per = (nchunks + g.ksplit - 1) / g.ksplit;
    S = (nchunks + per - 1) / per;
    a.ksplit = S;
  } else {
    a.ksplit = 1;
    a.partial = nullptr;
  }
  dim3 grid((unsigned)((g.M + kBM - 1) / kBM), (unsigned)((g.N + kBN - 1) / kBN), (unsigned)S);
  tn_gemm_kernel<<<grid, 128, smem, s>>>(a);
  if (S > 1) {
    const int64_t n = (int64_t)g.M * g.N;
    splitk_reduce_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a.partial, S, g.M, g.N, g.C,
                                                                     g.ldc);
  }
  return cudaGetLastError();
}

}  // namespace photic
