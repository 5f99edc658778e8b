// Low-precision trailing update of the mixed-precision LU (the PDGEMM step of
// SRC/pdgetrf.f:288-290 with 16-bit operands):
//
//   C (m x n, FP32, column-major) -= (A16 * B16^T) .* 2^e[col]
//
// A16 (m x k) and B16 (n x k) are BF16 or FP16 operand buffers stored K-major
// (k contiguous), produced from the FP32 working matrix by lowp_pack_* below;
// e[col] is the per-column power-of-two exponent that brought column `col` of
// U12 into the 16-bit range. Products of 16-bit operands are exact in FP32 and
// are accumulated in FP32 in tensor memory.
//
// Blackwell-native structure, one 128 x 256 output tile per CTA (4 warps):
//   * warp 0 allocates 256 TMEM columns (the FP32 accumulator, lane = row);
//   * one thread issues TMA loads (cp.async.bulk.tensor, 128-byte swizzle) of
//     the 128x64 A and 256x64 B k-blocks into a 2- or 3-stage shared-memory ring,
//     completion tracked by mbarrier transaction counts;
//   * one thread issues tcgen05.mma.cta_group::1.kind::f16 (M=128, N=256,
//     K=16) per 16-wide k-slice and frees each stage with tcgen05.commit;
//   * all 4 warps read the accumulator back with tcgen05.ld (warp w owns TMEM
//     lanes 32w..32w+31), write -acc * 2^e for 32 columns at a time into the
//     (now idle) stage buffers, and one thread adds each 128 x 32 chunk into C
//     with a TMA reduce (cp.reduce.async.bulk.tensor .add, FP32), so the
//     read-modify-write of C happens in L2 without a load round trip per
//     element. When C's base or leading dimension does not meet the TMA
//     alignment rules (16-byte base, ldc a multiple of 4) the epilogue falls
//     back to coalesced loads and stores of C.
// Two variants: 2 stages with two CTAs per SM (the default), or 3 stages with one CTA per SM
// (each holding 256 of the SM's 512 TMEM columns) so that one tile's epilogue
// overlaps the other's main loop.
// Every mbarrier wait is bounded; on timeout the CTA records kFlagTimeout in
// the status word, drains what it issued, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include "common.cuh"
#include "sl_internal.h"
#include "tc_common.cuh"

namespace sl {
namespace {
using namespace tc;

constexpr int BM = 128;
constexpr int BN = 256;
constexpr int BK = 64;       // 64 x 16-bit = 128 bytes: one swizzle row
constexpr int A_STAGE_BYTES = BM * BK * 2;  // 16 KB
constexpr int B_STAGE_BYTES = BN * BK * 2;  // 32 KB
constexpr int TMEM_COLS = 256;
// Instruction descriptor for kind::f16: FP32 accumulator, A/B both BF16 or
// both FP16, both K-major, N = 256, M = 128.
__host__ __device__ constexpr uint32_t make_idesc(bool bf16) {
  return (1u << 4)                          // D format: F32
         | ((bf16 ? 1u : 0u) << 7)          // A format
         | ((bf16 ? 1u : 0u) << 10)         // B format
         | ((uint32_t)(BN >> 3) << 17)      // N / 8
         | ((uint32_t)(BM >> 4) << 24);     // M / 16
}

constexpr int kMaxStages = 3;
struct __align__(8) GemmSmemTail {
  uint64_t full[kMaxStages];
  uint64_t empty[kMaxStages];
  uint64_t done;
  uint32_t tmem_base;
};

constexpr int EPI_COLS = 32;                       // columns per epilogue chunk
constexpr int EPI_CHUNK_BYTES = BM * EPI_COLS * 4;  // 16 KB staging per chunk

template <int STAGES, int MINB>
__global__ void __launch_bounds__(128, MINB)
lowp_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                 const __grid_constant__ CUtensorMap tmC, int use_tma_c, float* C, long long ldc,
                 int m, int n, int k, const int* __restrict__ col_exp, uint32_t idesc,
                 int* status) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // 1024-byte alignment for the swizzled stages
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = base;
  unsigned char* sB = base + STAGES * A_STAGE_BYTES;
  GemmSmemTail* tail = (GemmSmemTail*)(sB + STAGES * B_STAGE_BYTES);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int nk = (k + BK - 1) / BK;
  __shared__ int s_fail;
  __shared__ int s_issued, s_consumed;

  if (threadIdx.x == 0) {
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&tail->full[s], 1);
      mbar_init(&tail->empty[s], 1);
    }
    mbar_init(&tail->done, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tail->tmem_base)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tail->tmem_base;

  if (warp == 0 && lane == 0) {
    // TMA producer
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
    if (use_tma_c)
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmC)) : "memory");
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % STAGES;
      if (kb >= STAGES && !mbar_wait(&tail->empty[s], ((kb / STAGES) - 1) & 1)) {
        atomicExch(status, (int)kFlagTimeout);
        s_fail = 1;
        break;
      }
      mbar_expect_tx(&tail->full[s], A_STAGE_BYTES + B_STAGE_BYTES);
      tma_load_2d(sA + s * A_STAGE_BYTES, &tmA, &tail->full[s], kb * BK, m0);
      tma_load_2d(sB + s * B_STAGE_BYTES, &tmB, &tail->full[s], kb * BK, n0);
      s_issued = kb + 1;
    }
  } else if (warp == 1 && lane == 0) {
    // MMA issuer
    for (int kb = 0; kb < nk; ++kb) {
      const int s = kb % STAGES;
      if (!mbar_wait(&tail->full[s], (kb / STAGES) & 1)) {
        atomicExch(status, (int)kFlagTimeout);
        s_fail = 1;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int kk = 0; kk < BK / 16; ++kk) {
        uint64_t ad = smem_desc_sw128(sA + s * A_STAGE_BYTES + kk * 32);
        uint64_t bd = smem_desc_sw128(sB + s * B_STAGE_BYTES + kk * 32);
        umma_f16(tmem, ad, bd, idesc, (kb > 0 || kk > 0) ? 1u : 0u);
      }
      umma_commit(&tail->empty[s]);
      s_consumed = kb + 1;
    }
    umma_commit(&tail->done);  // arrives when every issued MMA has completed
  }
  __syncwarp();
  // Epilogue: all warps wait for the accumulator.
  bool ok = mbar_wait(&tail->done, 0);
  if (!ok) atomicExch(status, (int)kFlagTimeout);
  asm volatile("tcgen05.fence::after_thread_sync;");
  __syncthreads();
  if (ok && !s_fail && use_tma_c) {
    // Stage buffers are idle once every MMA has completed: reuse them as a
    // ring of 16 KB chunks, [column][row] FP32 (the TMA box's layout).
    constexpr int NSTG = STAGES * (A_STAGE_BYTES + B_STAGE_BYTES) / EPI_CHUNK_BYTES;
    static_assert(NSTG >= 2, "staging ring");
    const int rloc = warp * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c = 0; c < BN / EPI_COLS; ++c) {
      const int cb = n0 + c * EPI_COLS;
      if (cb >= n) break;  // uniform across the CTA
      float* stg = reinterpret_cast<float*>(base + (size_t)(c % NSTG) * EPI_CHUNK_BYTES);
      if (c >= NSTG) {
        // the reduce that last read this chunk must have finished reading it
        if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(NSTG - 1) : "memory");
        __syncthreads();
      }
      float v[32];
      tmem_ld32(trow + (uint32_t)(c * EPI_COLS), v);
      const int ncol = min(EPI_COLS, n - cb);
#pragma unroll
      for (int j = 0; j < EPI_COLS; ++j) {
        const float sc = (j < ncol) ? ldexpf(1.0f, __ldg(col_exp + cb + j)) : 0.f;
        stg[j * BM + rloc] = -v[j] * sc;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (threadIdx.x == 0) {
        tma_reduce_add_2d(&tmC, stg, m0, cb);  // rows >= m and columns >= n are clipped
        asm volatile("cp.async.bulk.commit_group;" ::: "memory");
      }
    }
    if (threadIdx.x == 0) asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
  } else if (ok && !s_fail) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 32) {
      if (n0 + c0 >= n) break;  // warp-uniform
      float v[32];
      tmem_ld32(trow + (uint32_t)c0, v);
      const int ncol = min(32, n - (n0 + c0));
      // Batch the 32 column scales and the 32 C loads before any store so the
      // loads are in flight together.
      float cv[32], sc[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) sc[j] = (j < ncol) ? ldexpf(1.0f, __ldg(col_exp + n0 + c0 + j)) : 0.f;
      float* cbase = C + (long long)row + (long long)(n0 + c0) * ldc;
      if (row < m) {
#pragma unroll
        for (int j = 0; j < 32; ++j) cv[j] = (j < ncol) ? cbase[(long long)j * ldc] : 0.f;
#pragma unroll
        for (int j = 0; j < 32; ++j)
          if (j < ncol) cbase[(long long)j * ldc] = fmaf(-v[j], sc[j], cv[j]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (s_fail && threadIdx.x == 0) {
    // Drain TMA copies that were issued but never consumed (bounded waits).
    for (int kb = s_consumed; kb < s_issued; ++kb)
      mbar_wait(&tail->full[kb % STAGES], (kb / STAGES) & 1);
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS));
  }
}

// ---- operand packing (FP32 working matrix -> 16-bit K-major operands) ------

__device__ __forceinline__ unsigned short bf16_hi(float x) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ unsigned short bf16_lo(float x) {
  float hi = __bfloat162float(__float2bfloat16_rn(x));
  return __bfloat16_as_ushort(__float2bfloat16_rn(x - hi));
}

template <bool BF16>
__device__ __forceinline__ unsigned short to16(float x) {
  if (BF16) return __bfloat16_as_ushort(__float2bfloat16_rn(x));
  return __half_as_ushort(__float2half_rn(x));
}

// A16[i*ldk + kk] = L21[i + kk*lda]  (m x k, transpose to K-major), kk < kpad
// zero-filled beyond k. 32x32 tiles through shared memory.
template <bool BF16>
__global__ void pack_a_kernel(const float* __restrict__ L, long long lda, int m, int k, int kpad,
                              unsigned short* A16) {
  __shared__ float t[32][33];
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    int kk = k0 + r, i = i0 + threadIdx.x;
    t[r][threadIdx.x] = (i < m && kk < k) ? L[i + (long long)kk * lda] : 0.f;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += 8) {
    int i = i0 + r, kk = k0 + threadIdx.x;
    if (i < m && kk < kpad) A16[(long long)i * kpad + kk] = to16<BF16>(t[threadIdx.x][r]);
  }
}

// Split packing for the 3-term BF16 product (fmt "bf16x3"): with x = hi + lo
// (both BF16), A*B ~= Ahi*Bhi + Ahi*Blo + Alo*Bhi, formed by one GEMM over a
// K dimension of 3*kpad: A3 = [Ahi | Ahi | Alo], B3 = [Bhi | Blo | Bhi].
__global__ void pack_a3_kernel(const float* __restrict__ L, long long lda, int m, int k, int kpad,
                               unsigned short* A3) {
  __shared__ float t[32][33];
  const int i0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += 8) {
    int kk = k0 + r, i = i0 + threadIdx.x;
    t[r][threadIdx.x] = (i < m && kk < k) ? L[i + (long long)kk * lda] : 0.f;
  }
  __syncthreads();
  const long long ld3 = 3LL * kpad;
  for (int r = threadIdx.y; r < 32; r += 8) {
    int i = i0 + r, kk = k0 + threadIdx.x;
    if (i < m && kk < kpad) {
      float x = t[threadIdx.x][r];
      unsigned short h = bf16_hi(x), l = bf16_lo(x);
      A3[(long long)i * ld3 + kk] = h;
      A3[(long long)i * ld3 + kpad + kk] = h;
      A3[(long long)i * ld3 + 2 * kpad + kk] = l;
    }
  }
}

__global__ void pack_b3_kernel(const float* __restrict__ U, long long ldu, int k, int n, int kpad,
                               unsigned short* B3, int* col_exp) {
  const int j = blockIdx.x;
  if (j >= n) return;
  __shared__ float s_max[32];
  float mx = 0.f;
  for (int kk = threadIdx.x; kk < k; kk += blockDim.x) mx = fmaxf(mx, fabsf(U[kk + (long long)j * ldu]));
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    mx = threadIdx.x < (blockDim.x >> 5) ? s_max[threadIdx.x] : 0.f;
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if (threadIdx.x == 0) {
      int e = 0;
      if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
      s_max[0] = __int_as_float(e);
    }
  }
  __syncthreads();
  const int e = __float_as_int(s_max[0]);
  if (threadIdx.x == 0) col_exp[j] = e;
  const float sc = ldexpf(1.0f, -e);
  const long long ld3 = 3LL * kpad;
  for (int kk = threadIdx.x; kk < kpad; kk += blockDim.x) {
    float x = kk < k ? U[kk + (long long)j * ldu] * sc : 0.f;
    unsigned short h = bf16_hi(x), l = bf16_lo(x);
    B3[(long long)j * ld3 + kk] = h;
    B3[(long long)j * ld3 + kpad + kk] = l;
    B3[(long long)j * ld3 + 2 * kpad + kk] = h;
  }
}

// Per-column exponent of U12 (k x n, column-major): e[j] = exponent that
// scales max|U12[:,j]| into [0.5, 1); B16[j*kpad + kk] = U12[kk + j*ldu] * 2^-e.
template <bool BF16>
__global__ void pack_b_kernel(const float* __restrict__ U, long long ldu, int k, int n, int kpad,
                              unsigned short* B16, int* col_exp) {
  const int j = blockIdx.x;
  if (j >= n) return;
  __shared__ float s_max[32];
  float mx = 0.f;
  for (int kk = threadIdx.x; kk < k; kk += blockDim.x) mx = fmaxf(mx, fabsf(U[kk + (long long)j * ldu]));
  for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    mx = threadIdx.x < (blockDim.x >> 5) ? s_max[threadIdx.x] : 0.f;
    for (int off = 16; off > 0; off >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    if (threadIdx.x == 0) {
      int e = 0;
      if (mx > 0.f && isfinite(mx)) frexpf(mx, &e);
      s_max[0] = __int_as_float(e);
    }
  }
  __syncthreads();
  const int e = __float_as_int(s_max[0]);
  if (threadIdx.x == 0) col_exp[j] = e;
  const float sc = ldexpf(1.0f, -e);
  for (int kk = threadIdx.x; kk < kpad; kk += blockDim.x)
    B16[(long long)j * kpad + kk] = to16<BF16>(kk < k ? U[kk + (long long)j * ldu] * sc : 0.f);
}

// 2D tensor map over a rows x kpad row-major 16-bit operand, box {64, box_rows}.
bool make_map(CUtensorMap* map, const void* ptr, int rows, int kpad, int box_rows) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)kpad * 2};
  cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 2, const_cast<void*>(ptr), dims, strides,
                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// 2D tensor map over C (m x n FP32, column-major, leading dimension ldc) with a
// 128 x 32 box for the epilogue's reduce; false when C does not meet the TMA
// rules (16-byte base, 16-byte multiple stride).
bool make_map_c(CUtensorMap* map, float* C, int m, int n, long long ldc) {
  if ((reinterpret_cast<uintptr_t>(C) & 15) != 0 || (ldc & 3) != 0) return false;
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)m, (cuuint64_t)n};
  cuuint64_t strides[1] = {(cuuint64_t)ldc * 4};
  cuuint32_t box[2] = {(cuuint32_t)BM, (cuuint32_t)EPI_COLS};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, C, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

int g_lowp_stages = 2;  // 2: two CTAs per SM (default); 3: one CTA per SM

// Raises the kernel's dynamic shared-memory limit once per instantiation.
template <int ST, int MB>
cudaError_t smem_limit_once(size_t bytes) {
  static const cudaError_t e = cudaFuncSetAttribute(
      lowp_gemm_kernel<ST, MB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return e;
}

size_t smem_bytes_for(int stages) {
  return 1024 + (size_t)stages * (A_STAGE_BYTES + B_STAGE_BYTES) + sizeof(GemmSmemTail) + 64;
}

}  // namespace

size_t lowp_gemm_smem_bytes() { return smem_bytes_for(g_lowp_stages); }

void lowp_set_stages(int stages) { g_lowp_stages = (stages == 2) ? 2 : 3; }

int lowp_kpad(int k) { return (k + BK - 1) / BK * BK; }

int lowp_kmult(int fmt) { return fmt == 2 ? 3 : 1; }

cudaError_t lowp_pack(int fmt, const float* L, long long lda, int m, const float* U,
                      long long ldu, int n, int k, unsigned short* A16, unsigned short* B16,
                      int* col_exp, cudaStream_t s) {
  const int kpad = lowp_kpad(k);
  if (fmt == 2) {
    if (m > 0) {
      dim3 g((m + 31) / 32, (kpad + 31) / 32), b(32, 8);
      pack_a3_kernel<<<g, b, 0, s>>>(L, lda, m, k, kpad, A16);
      count_launches(1);
    }
    if (n > 0) {
      pack_b3_kernel<<<n, 128, 0, s>>>(U, ldu, k, n, kpad, B16, col_exp);
      count_launches(1);
    }
    return cudaGetLastError();
  }
  const bool bf16 = (fmt == 0);
  if (m > 0) {
    dim3 g((m + 31) / 32, (kpad + 31) / 32), b(32, 8);
    if (bf16) pack_a_kernel<true><<<g, b, 0, s>>>(L, lda, m, k, kpad, A16);
    else pack_a_kernel<false><<<g, b, 0, s>>>(L, lda, m, k, kpad, A16);
    count_launches(1);
  }
  if (n > 0) {
    if (bf16) pack_b_kernel<true><<<n, 128, 0, s>>>(U, ldu, k, n, kpad, B16, col_exp);
    else pack_b_kernel<false><<<n, 128, 0, s>>>(U, ldu, k, n, kpad, B16, col_exp);
    count_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t lowp_gemm(int fmt, int m, int n, int k, const unsigned short* A16,
                      const unsigned short* B16, const int* col_exp, float* C, long long ldc,
                      int* status, cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  const bool bf16 = (fmt != 1);
  const int kpad = lowp_kpad(k) * lowp_kmult(fmt);
  CUtensorMap ta, tb, tc;
  if (!make_map(&ta, A16, m, kpad, BM) || !make_map(&tb, B16, n, kpad, BN))
    return cudaErrorInvalidResourceHandle;
  const int use_tma_c = make_map_c(&tc, C, m, n, ldc) ? 1 : 0;
  if (!use_tma_c) tc = ta;  // unused by the kernel
  dim3 grid((m + BM - 1) / BM, (n + BN - 1) / BN);
  const uint32_t idesc = make_idesc(bf16);
  if (g_lowp_stages == 2) {
    const size_t smem = smem_bytes_for(2);
    SL_TRY((smem_limit_once<2, 2>(smem)));
    lowp_gemm_kernel<2, 2><<<grid, 128, smem, s>>>(ta, tb, tc, use_tma_c, C, ldc, m, n, kpad,
                                                   col_exp, idesc, status);
  } else {
    const size_t smem = smem_bytes_for(3);
    SL_TRY((smem_limit_once<3, 1>(smem)));
    lowp_gemm_kernel<3, 1><<<grid, 128, smem, s>>>(ta, tb, tc, use_tma_c, C, ldc, m, n, kpad,
                                                   col_exp, idesc, status);
  }
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace sl
