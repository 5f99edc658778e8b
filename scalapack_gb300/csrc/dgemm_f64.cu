// FP64 GEMM for the PDGEMM trailing update (SRC/pdgetrf.f:288-290, which on a
// 1x1 grid is one local DGEMM: PBLAS/SRC/PTOOLS/PB_CpgemmAB.c:333-351).
//
// sm_103a has no FP64 tcgen05 kind; FP64 tensor math is the DMMA
// mma.sync.m16n8k4.f64 path. On GB300 the FP64 pipe is narrow (about
// 1.05 TFLOP/s for both DMMA and DFMA across 152 SMs), so this kernel is
// compute-bound by a wide margin: a 128x128x16 stage is ~164k SM cycles of DMMA
// work but only 37 KB of loads. The design goals are therefore (1) never starve
// the DMMA issue (two-stage cp.async pipeline, 8 warps x 16 independent
// accumulator tiles) and (2) keep every SM busy (tile size chosen per shape).
//
// C (m x n) = alpha * op(A) (m x k) * B (k x n) + beta * C, column-major.
#include <cuda_runtime.h>

#include <atomic>
#include <stdint.h>
#include "common.cuh"
#include "sl_internal.h"

namespace sl {

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool pred) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  int sz = pred ? 8 : 0;  // src-size 0 => the 8 destination bytes are zero-filled
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(s), "l"(gmem), "r"(sz));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N)); }

__device__ __forceinline__ void dmma_16x8x4(double* c, double a0, double a1, double b0) {
  asm volatile(
      "mma.sync.aligned.m16n8k4.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5}, {%6}, "
      "{%0,%1,%2,%3};"
      : "+d"(c[0]), "+d"(c[1]), "+d"(c[2]), "+d"(c[3])
      : "d"(a0), "d"(a1), "d"(b0));
}

// Block tile BM x BN, K-step 16, warps arranged WM x WN; each warp owns a
// (BM/WM) x (BN/WN) sub-tile made of m16n8 DMMA tiles.
// Shared layouts (bank-conflict free for the fragment reads):
//   As[k][m] with row stride BM+4 doubles, Bs[n][k] with row stride 20.
template <int BM, int BN, int WM, int WN, bool TRANSA>
__global__ void __launch_bounds__(WM* WN * 32)
dgemm_dmma_kernel(int m, int n, int k, double alpha, const double* __restrict__ A, long long lda,
                  const double* __restrict__ B, long long ldb, double beta, double* C,
                  long long ldc) {
  constexpr int BK = 16;
  constexpr int NT = WM * WN * 32;
  constexpr int LDA_S = BM + 4;
  constexpr int LDB_S = BK + 4;
  constexpr int TM = BM / WM / 16;  // m16 tiles per warp
  constexpr int TN = BN / WN / 8;   // n8 tiles per warp
  extern __shared__ __align__(16) double smem[];
  double* As = smem;                       // [2][BK][LDA_S]
  double* Bs = smem + 2 * BK * LDA_S;      // [2][BN][LDB_S]

  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int wm = warp % WM, wn = warp / WM;
  const long long m0 = (long long)blockIdx.x * BM;
  const long long n0 = (long long)blockIdx.y * BN;

  double acc[TM][TN][4];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0;

  auto load_stage = [&](int stage, int k0) {
    double* as = As + stage * BK * LDA_S;
    double* bs = Bs + stage * BN * LDB_S;
    // A tile: BM x BK of op(A)
#pragma unroll
    for (int c = tid; c < BM * BK; c += NT) {
      int mm, kk;
      if (!TRANSA) { kk = c / BM; mm = c % BM; }   // consecutive threads -> consecutive m
      else { mm = c / BK; kk = c % BK; }           // consecutive threads -> consecutive k
      long long gm = m0 + mm, gk = k0 + kk;
      bool ok = (gm < m) && (gk < k);
      const double* src = ok ? (TRANSA ? A + gk + gm * lda : A + gm + gk * lda) : A;
      cp_async8(as + kk * LDA_S + mm, src, ok);
    }
    // B tile: BK x BN
#pragma unroll
    for (int c = tid; c < BN * BK; c += NT) {
      int nn = c / BK, kk = c % BK;
      long long gn = n0 + nn, gk = k0 + kk;
      bool ok = (gn < n) && (gk < k);
      const double* src = ok ? B + gk + gn * ldb : B;
      cp_async8(bs + nn * LDB_S + kk, src, ok);
    }
  };

  const int ktiles = (k + BK - 1) / BK;
  if (ktiles > 0) {
    load_stage(0, 0);
    cp_async_commit();
  }
  for (int kt = 0; kt < ktiles; ++kt) {
    if (kt + 1 < ktiles) load_stage((kt + 1) & 1, (kt + 1) * BK);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const double* as = As + (kt & 1) * BK * LDA_S;
    const double* bs = Bs + (kt & 1) * BN * LDB_S;
#pragma unroll
    for (int kk = 0; kk < BK; kk += 4) {
      double a0[TM], a1[TM], b0[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) {
        int mrow = wm * (BM / WM) + i * 16 + g;
        a0[i] = as[(kk + t) * LDA_S + mrow];
        a1[i] = as[(kk + t) * LDA_S + mrow + 8];
      }
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        int ncol = wn * (BN / WN) + j * 8 + g;
        b0[j] = bs[ncol * LDB_S + kk + t];
      }
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) dmma_16x8x4(acc[i][j], a0[i], a1[i], b0[j]);
    }
    __syncthreads();
  }

  // Epilogue: C = alpha*acc + beta*C
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        long long row = m0 + wm * (BM / WM) + i * 16 + g + ((r & 2) ? 8 : 0);
        long long col = n0 + wn * (BN / WN) + j * 8 + 2 * t + (r & 1);
        if (row < m && col < n) {
          double* cp = C + row + col * ldc;
          double v = alpha * acc[i][j][r];
          *cp = (beta == 0.0) ? v : fma(beta, *cp, v);
        }
      }
}

template <int BM, int BN, int WM, int WN, bool TA>
static cudaError_t launch_dmma(int m, int n, int k, double alpha, const double* A, long long lda,
                               const double* B, long long ldb, double beta, double* C,
                               long long ldc, cudaStream_t s) {
  constexpr int BK = 16;
  size_t smem = sizeof(double) * (2 * BK * (BM + 4) + 2 * BN * (BK + 4));
  auto kern = dgemm_dmma_kernel<BM, BN, WM, WN, TA>;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid((m + BM - 1) / BM, (n + BN - 1) / BN);
  kern<<<grid, WM * WN * 32, smem, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  count_launches(1);
  return cudaGetLastError();
}

// Number of SMs of the current device, cached per device; 1 while no device
// answers (not cached, so a later call on a working device gets its count).
int num_sms() {
  constexpr int kDevs = 64;
  static std::atomic<int> cache[kDevs];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  if (dev >= 0 && dev < kDevs) {
    const int c = cache[dev].load(std::memory_order_relaxed);
    if (c > 0) return c;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return 1;
  }
  if (dev >= 0 && dev < kDevs) cache[dev].store(n, std::memory_order_relaxed);
  return n;
}

cudaError_t dgemm(bool transa, int m, int n, int k, double alpha, const double* A, long long lda,
                  const double* B, long long ldb, double beta, double* C, long long ldc,
                  cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  if (k <= 0) {
    if (beta == 1.0) return cudaSuccess;
  }
  // Pick the tile so that the grid covers the SMs: 128x128 when there are at
  // least ~2 waves of big tiles, 64x64 otherwise.
  long long big_tiles = (long long)((m + 127) / 128) * ((n + 127) / 128);
  if (big_tiles >= 2LL * num_sms()) {
    if (transa) return launch_dmma<128, 128, 2, 4, true>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
    return launch_dmma<128, 128, 2, 4, false>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
  }
  if (transa) return launch_dmma<64, 64, 2, 2, true>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
  return launch_dmma<64, 64, 2, 2, false>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, s);
}

// FP64 tensor peak calibration: every warp issues independent chains of
// m16n8k4 DMMA on register operands (no memory traffic), 2 CTAs x 8 warps per
// SM. The result bounds what any FP64 GEMM on this device can reach.
__global__ void __launch_bounds__(256) dmma_peak_kernel(double* out, int iters) {
  double c[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) c[i][j] = 0.0;
  double a0 = 1e-3 * threadIdx.x, a1 = 2e-3 * threadIdx.x, b0 = 1e-3 * (threadIdx.x + 1);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int ch = 0; ch < 8; ++ch) dmma_16x8x4(c[ch], a0, a1, b0);
  }
  double sum = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) sum += c[i][j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = sum;
}

double dmma_peak_tflops(cudaStream_t s) {
  const int blocks = 2 * num_sms(), threads = 256, iters = 4000;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * blocks * threads) != cudaSuccess) return 0.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0, s);
    dmma_peak_kernel<<<blocks, threads, 0, s>>>(d, iters);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  double flops = 2.0 * 16 * 8 * 4 * 8.0 * iters * (double)blocks * (threads / 32);
  return flops / (best * 1e-3) / 1e12;
}

}  // namespace sl
