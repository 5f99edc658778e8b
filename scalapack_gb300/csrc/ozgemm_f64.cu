// FP64 trailing update of the plain LU on the BF16 tensor cores (the PDGEMM
// step of SRC/pdgetrf.f:288-290, C <- C + alpha * A * B with FP64 A, B, C):
// sm_103a's tcgen05.mma has no FP64 kind, so the product is formed exactly
// from integer slices (the error-free splitting of Ozaki, Ogita and Oishi,
// "Error-free transformations of matrix multiplication by using fast routines
// of matrix multiplication and its applications", Numer. Algorithms 59, 2012).
//
// Splitting. Row i of A is scaled by 2^-e_i (e_i the exponent of its largest
// magnitude, so |A(i,k)| 2^-e_i < 1) and cut into S = 8 slices of 7 bits:
//   A(i,k) 2^-e_i = sum_{s=1..8} a_s(i,k) 2^-7s,  a_s integer, |a_s| <= 127,
// by exact FP64 truncation; column j of B likewise with 2^-f_j and b_t. The
// slices are stored in BF16 as a_s 2^-7(s-1) (8 significant bits hold any
// |a_s| <= 127 and the power of two is exact), K-major, so that the product of
// slices s and t carries its weight 2^-7(s+t-2) by itself.
//
// Exact products. For K <= 256, sum_k a_s b_t is an integer of magnitude at
// most 256 * 127^2 < 2^22: up to four such products sum exactly in FP32, in
// any order and with any alignment the tensor core uses, because every partial
// sum is an integer multiple of the diagonal's unit below 2^24. With
// d = s + t, the update is
//   (A B)(i,j) = 2^(e_i + f_j) sum_d 2^-7d P_d,   P_d = sum_{s+t=d} sum_k a_s b_t.
// Each diagonal d = 2..9 has its own TMEM accumulator (8 x 64 columns, all of
// TMEM). d <= 5 holds at most 4 products: exact; d = 6 holds 5, exact unless
// their sum passes 2^24, which takes nearly all 1280 terms at full magnitude
// with one sign; d = 7..9 are summed in plain FP32 (their rounding, 2^-24
// relative to terms already 2^-49 below the row and column scales, is far
// below FP64 rounding); d >= 10 is dropped. 36 slice products, issued as 12
// instructions per 16-wide k step: A slice s against B slices t = 0..7-s
// (consecutive in shared memory) into accumulators s..7 (consecutive in TMEM)
// in groups of up to 4 (N up to 256).
//
// Epilogue. P_2..P_6 are read back as exact integers, combined with the FP32
// sum of the tail diagonals into one 64-bit integer I = sum_d P_d 2^(52-7d) (|I| < 2^61), converted to
// FP64 once, and C(i,j) = fma(alpha 2^(e_i+f_j-52), I, C(i,j)). The result is
// within a few units of 2^-53 of 2^(e_i + f_j) of the exact product, and
// independent of the accumulation order (run to run identical). Rows or
// columns holding Inf or NaN give NaN in their row or column of C.
//
// Balancing along k. A B = (A 2^-d)(2^d B) for any integers d_k, so the
// scales are taken after an exact power-of-two balancing (ex x: |x| < 2^ex x,
// over the k whose column of A and row of B are both nonzero):
//   e_i = max_k (ex A(i,k) - d_k),   f_j = max_k (ex B(k,j) + d_k).
// The shift goes into the slicing's shift counts; no scaled value is ever
// formed. Side A (the default): d_k = c_k, the exponent of the largest
// magnitude in column k of A. In the LU A = L21 (|L| <= 1, so c_k ~ 0 and
// nothing moves on well-scaled data); on a row-graded matrix a block's pivots
// differ widely in size, column k of L21 is ~2^-(s_pk) and row k of U12
// ~2^(s_pk), and without the balancing the largest L21 and U12 entries of a
// pair (i, j) sit at different k, so 2^(e_i + f_j) would exceed every term of
// the product by the pivots' spread. Side B: d_k = -h_k, h_k the exponent of
// the largest magnitude in row k of B -- for the U12 solve's product
// (inv(L_bb) - I) A12_b, whose rows of B carry the pivots' scales while the
// columns of the inverse do not.
//
// Error budget. With G = max_k (c_k + h_k), side A compares each row's error
// bound 2^(e_i + G) with F_i = max_k (ex A(i,k) + h_k), the exponent of a
// lower bound of max_j (|A| |B|)(i,j) (an FP64 GEMM's bound for that row);
// side B compares each column's 2^(f_j + G) with F_j = max_k (c_k +
// ex B(k,j)). Where any row (column) is more than OZ_BUDGET bits above it (a
// row of A small exactly where a row of B holds an entry far above the rest),
// or a scale leaves the normal FP64 range, the whole pass is computed in FP64
// arithmetic instead (fixed order, every product an FMA) by the same
// launches. Accuracy model: each row's (column's) error is within about
// 2^OZ_BUDGET of the FP64 GEMM's error bound for its largest |A||B| term
// (normwise per row or column); for inputs that are diagonal scalings of
// well-scaled data that is the componentwise level. Operands whose large
// entries cross (row i large at k1 only, column j large at k2 only) keep the
// normwise bound but not a componentwise one.
//
// Structure (one CTA per SM, a few 128 x 64 tiles of C per CTA, 10 warps):
//   * warp 0 allocates all 512 TMEM columns (8 accumulators x 64 columns);
//   * one thread issues TMA loads: for each 64-wide k block, the eight 128x64
//     A slices one at a time through a 6-deep ring and the eight 64x64 B
//     slices into one half of a double buffer, half a block ahead (128-byte
//     swizzle);
//   * one thread issues tcgen05.mma.kind::f16 (M=128, N=64..256, K=16): A
//     slice s against B slices t <= 9 - s into accumulators s+t-2;
//   * 8 epilogue warps read the accumulators with tcgen05.ld (warp w owns
//     lanes 32(w%4).. = tile rows, and half of the columns), combine them
//     into integers, hand the TMEM
//     back to the MMA thread, and update C in place (coalesced per column)
//     while the next tile's products run.
// Every mbarrier wait is bounded; on timeout the CTA records kFlagTimeout,
// drains what it issued, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <climits>

#include "common.cuh"
#include "sl_internal.h"
#include "tc_common.cuh"

namespace sl {
namespace {
using namespace tc;

constexpr int OZ_S = 8;          // slices per operand
constexpr int OZ_BITS = 7;       // bits per slice
constexpr int OZ_NACC = 8;       // accumulators, one per diagonal d = 2..9
constexpr int OZ_KMAX = 256;     // exactness bound on K per pass
constexpr int OBM = 128, OBN = 64, OBK = 64;
constexpr int A_SLICE_BYTES = OBM * OBK * 2;          // 16 KB
constexpr int B_SLICE_BYTES = OBN * OBK * 2;          // 8 KB
constexpr int B_CHUNK_BYTES = OZ_S * B_SLICE_BYTES;   // 64 KB per k block
constexpr int A_RING = 6;
constexpr int OZ_TMEM_COLS = 512;
constexpr int GROUP_M = 8;       // tile raster: 8 row tiles sweep the columns together

// Balancing / budget area at the start of the scratch: h keys [256] (rows of
// B), c keys [256] (columns of A), the FP64-route flag. Each word is
// (epoch << 12) | (exponent + OZ_EBIAS), so a pass ignores what earlier passes
// left (epochs only grow) and nothing has to be cleared between passes.
constexpr int OZ_KINFO_BYTES = kOzKinfoBytes;
constexpr int OZ_KI_H = 0, OZ_KI_C = OZ_KMAX, OZ_KI_FLAG = 2 * OZ_KMAX;
constexpr int OZ_EBIAS = kOzEbias;
constexpr int OZ_BUDGET = 8;     // bits above the FP64 GEMM's row (column) bound
constexpr int OZ_NOEXP = INT_MIN / 4;

__device__ unsigned long long g_oz_fp64_routes;  // passes that took the FP64 route

struct __align__(8) OzBars {
  uint64_t afull[A_RING], aempty[A_RING];
  uint64_t bfull[2], bempty[2];
  uint64_t tfull, tempty;  // accumulators complete / drained
  uint32_t tmem_base;
};

constexpr int OZ_THREADS = 320;  // warp 0 TMA, warp 1 MMA, warps 2..9 epilogue
constexpr int OZ_EPI_WARPS = 8;  // two per TMEM lane quadrant, 32 columns each

size_t oz_smem_bytes() {
  return 1024 + (size_t)A_RING * A_SLICE_BYTES + 2 * (size_t)B_CHUNK_BYTES + sizeof(OzBars) + 64;
}

// kind::f16 instruction descriptor, M = 128, N = nn (a multiple of 64 <= 256)
__host__ __device__ constexpr uint32_t oz_idesc(int nn) {
  return (1u << 4)                       // D format: F32
         | (1u << 7) | (1u << 10)        // A, B: BF16
         | ((uint32_t)(nn >> 3) << 17)   // N / 8
         | ((uint32_t)(OBM >> 4) << 24); // M / 16
}

__device__ __forceinline__ void touch16(uint32_t* r) {
  asm volatile(""
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]),
                 "+r"(r[6]), "+r"(r[7]), "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]),
                 "+r"(r[12]), "+r"(r[13]), "+r"(r[14]), "+r"(r[15]));
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Tile t of the grouped raster: (m0, n0).
__device__ __forceinline__ void oz_tile(int t, int tiles_m, int tiles_n, int& m0, int& n0) {
  const int per_group = GROUP_M * tiles_n;
  const int gid = t / per_group, first_m = gid * GROUP_M;
  const int gsize = min(tiles_m - first_m, GROUP_M);
  const int in_group = t % per_group;
  m0 = (first_m + in_group % gsize) * OBM;
  n0 = (in_group / gsize) * OBN;
}

// The eight B slices of chunk c (tile first + c / nkc, k block c % nkc) into
// half c & 1 of the B double buffer, once chunk c-2 has released it.
__device__ __forceinline__ bool oz_issue_b(int c, int first, int nkc, int tiles_m, int tiles_n,
                                           int n_pad, unsigned char* sB, const CUtensorMap* tmB,
                                           OzBars* bars, int* issued) {
  const int hb = c & 1;
  if (c >= 2 && !mbar_wait(&bars->bempty[hb], ((c >> 1) - 1) & 1)) return false;
  int m0, n0;
  oz_tile(first + c / nkc, tiles_m, tiles_n, m0, n0);
  const int kc = c % nkc;
  mbar_expect_tx(&bars->bfull[hb], B_CHUNK_BYTES);
  for (int t = 0; t < OZ_S; ++t)
    tma_load_2d(sB + hb * B_CHUNK_BYTES + t * B_SLICE_BYTES, tmB, &bars->bfull[hb], kc * OBK,
                t * n_pad + n0);
  *issued = c + 1;
  return true;
}

// The FP64 route of a pass whose slices would exceed the error budget: the
// CTA's tiles computed directly from the FP64 operands. B's 64 columns of a
// tile (kb <= 256 rows, 128 KB) are staged in shared memory before any of
// them is written. When B aliases C (whole_cols) a CTA takes whole column
// blocks instead -- tile t of the CTA is column block t with every row tile --
// so no other CTA writes the columns it reads. Threads 64.. own one row and
// 32 columns each; products accumulate in k order with one FMA each, then
// C = fma(alpha, acc, C).
__device__ __noinline__ void oz_fp64_tiles(unsigned char* smem, int m, int n, int kb,
                                           const double* __restrict__ A, long long lda,
                                           const double* B, long long ldb, double alpha,
                                           double* C, long long ldc, int first_tile,
                                           int my_tiles, int tiles_m, int tiles_n,
                                           int whole_cols) {
  double* sB = reinterpret_cast<double*>(smem);  // [kb][64]
  const int tid = threadIdx.x;
  const int nsub = whole_cols ? tiles_m : 1;
  for (int it = 0; it < my_tiles * nsub; ++it) {
    int m0, n0;
    if (whole_cols) {
      const int t = first_tile + it / nsub;
      if (t >= tiles_n) break;
      n0 = t * OBN;
      m0 = (it % nsub) * OBM;
    } else {
      oz_tile(first_tile + it, tiles_m, tiles_n, m0, n0);
    }
    __syncthreads();
    if (!whole_cols || (it % nsub) == 0)
      for (int idx = tid; idx < kb * OBN; idx += OZ_THREADS) {
        const int c = idx / kb, k = idx - c * kb;
        sB[k * OBN + c] = (n0 + c < n) ? B[k + (long long)(n0 + c) * ldb] : 0.0;
      }
    __syncthreads();
    if (tid >= 64) {
      const int t = tid - 64, row = m0 + (t & (OBM - 1)), h = t >> 7;
      if (row < m) {
        double acc[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[j] = 0.0;
        const double* arow = A + row;
        for (int k = 0; k < kb; ++k) {
          const double a = arow[(long long)k * lda];
          const double* bk = sB + k * OBN + h * 32;
#pragma unroll
          for (int j = 0; j < 32; ++j) acc[j] = fma(a, bk[j], acc[j]);
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int col = n0 + h * 32 + j;
          if (col < n) {
            double* cp = C + row + (long long)col * ldc;
            *cp = fma(alpha, acc[j], *cp);
          }
        }
      }
    }
  }
}

// CTA b takes tiles b tpc .. b tpc + tpc - 1 of the raster (a few, so that
// SMs turn over and the panel's kernels on the high-priority stream find
// room between them). The TMA thread runs
// ahead through a flat sequence of k blocks ("chunks", nkc per tile): for
// chunk c it loads the eight A slices through the ring, and after the fourth
// of them the eight B slices of chunk c+1 into the other half of the B double
// buffer. The MMA thread starts a tile once the epilogue has drained the
// previous tile's accumulators (tempty); the epilogue warps drain them into
// 32 combined integers per thread (tmem -> registers), release the TMEM, and
// update C from registers while the next tile's products run.
__global__ void __launch_bounds__(OZ_THREADS, 1)
ozgemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
              int m, int n, int kpad, int m_pad, int n_pad, const double* __restrict__ rs,
              const double* __restrict__ cs, double alpha, double* C, long long ldc, int tpc,
              int* status, const double* __restrict__ A64, long long lda, const double* B64,
              long long ldb, int kb, const unsigned long long* kinfo, unsigned long long epoch) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  unsigned char* sA = base;                                   // A_RING x 16 KB
  unsigned char* sB = base + A_RING * A_SLICE_BYTES;          // 2 x 64 KB
  OzBars* bars = (OzBars*)(sB + 2 * B_CHUNK_BYTES);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_m = m_pad / OBM, tiles_n = n_pad / OBN;
  const int tiles = tiles_m * tiles_n;
  const int first_tile = (int)blockIdx.x * tpc;
  const int my_tiles = max(0, min(tpc, tiles - first_tile));
  const int nkc = kpad / OBK;
  const int total = my_tiles * nkc;  // chunks of this CTA
  __shared__ int s_fail, s_aiss, s_acons, s_biss, s_bcons;
  // a CTA that timed out already marked the launch failed: skip the work
  if (*(volatile int*)status != 0) return;
  // the slicing found the pass outside the error budget: FP64 route
  if (*(volatile const unsigned long long*)(kinfo + OZ_KI_FLAG) == epoch) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&g_oz_fp64_routes, 1ULL);
    oz_fp64_tiles(base, m, n, kb, A64, lda, B64, ldb, alpha, C, ldc, first_tile, my_tiles,
                  tiles_m, tiles_n, B64 == C ? 1 : 0);
    return;
  }

  if (threadIdx.x == 0) {
    s_fail = 0;
    s_aiss = s_acons = s_biss = s_bcons = 0;
    for (int i = 0; i < A_RING; ++i) {
      mbar_init(&bars->afull[i], 1);
      mbar_init(&bars->aempty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&bars->bfull[i], 1);
      mbar_init(&bars->bempty[i], 1);
    }
    mbar_init(&bars->tfull, 1);
    mbar_init(&bars->tempty, OZ_EPI_WARPS);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&bars->tmem_base)),
                 "r"(OZ_TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = bars->tmem_base;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer ----
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
      bool ok = total == 0 ||
                oz_issue_b(0, first_tile, nkc, tiles_m, tiles_n, n_pad, sB, &tmB, bars, &s_biss);
      for (int c = 0; ok && c < total; ++c) {
        int m0, n0;
        oz_tile(first_tile + c / nkc, tiles_m, tiles_n, m0, n0);
        const int kc = c % nkc;
        for (int sl = 0; ok && sl < OZ_S; ++sl) {
          const int g = c * OZ_S + sl, st = g % A_RING;
          if (g >= A_RING && !mbar_wait(&bars->aempty[st], ((g / A_RING) - 1) & 1)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&bars->afull[st], A_SLICE_BYTES);
          tma_load_2d(sA + st * A_SLICE_BYTES, &tmA, &bars->afull[st], kc * OBK, sl * m_pad + m0);
          s_aiss = g + 1;
          if (sl == 3 && c + 1 < total &&
              !oz_issue_b(c + 1, first_tile, nkc, tiles_m, tiles_n, n_pad, sB, &tmB, bars, &s_biss))
            ok = false;
        }
        if (s_fail) ok = false;
      }
      if (!ok) {
        atomicExch(status, (int)kFlagTimeout);
        s_fail = 1;
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      // A slice s against B slices t = 0 .. 7-s lands in accumulators s .. 7:
      // consecutive TMEM columns and, in the B buffer, consecutive slices, so
      // one instruction covers up to 4 of them (N up to 256).
      bool ok = true;
      for (int it = 0; ok && it < my_tiles; ++it) {
        if (it >= 1 && !mbar_wait(&bars->tempty, (it - 1) & 1)) { ok = false; break; }
        asm volatile("tcgen05.fence::after_thread_sync;");
        for (int kc = 0; ok && kc < nkc; ++kc) {
          const int c = it * nkc + kc, hb = c & 1;
          if (!mbar_wait(&bars->bfull[hb], (c >> 1) & 1)) { ok = false; break; }
          s_bcons = c + 1;
          const unsigned char* bchunk = sB + hb * B_CHUNK_BYTES;
          for (int sl = 0; sl < OZ_S; ++sl) {
            const int g = c * OZ_S + sl, st = g % A_RING;
            if (!mbar_wait(&bars->afull[st], (g / A_RING) & 1)) { ok = false; break; }
            asm volatile("tcgen05.fence::after_thread_sync;");
            const unsigned char* aslice = sA + st * A_SLICE_BYTES;
#pragma unroll
            for (int kk = 0; kk < OBK / 16; ++kk) {
              const uint64_t ad = smem_desc_sw128(aslice + kk * 32);
              // the very first products write every accumulator (s = 0 covers
              // all eight); every later one adds
              const uint32_t accum = (kc > 0 || sl > 0 || kk > 0) ? 1u : 0u;
              for (int t0 = 0; t0 + sl < OZ_S; t0 += 4) {
                const int cnt = min(4, OZ_S - sl - t0);
                const uint32_t dst = tmem + (uint32_t)((sl + t0) * OBN);
                const uint64_t bd = smem_desc_sw128(bchunk + t0 * B_SLICE_BYTES + kk * 32);
                umma_f16(dst, ad, bd, oz_idesc(cnt * OBN), accum);
              }
            }
            umma_commit(&bars->aempty[st]);
            s_acons = g + 1;
          }
          if (!ok) break;
          umma_commit(&bars->bempty[hb]);
        }
        if (ok) umma_commit(&bars->tfull);  // arrives when the tile's products are complete
        if (s_fail) ok = false;
      }
      if (!ok) {
        atomicExch(status, (int)kFlagTimeout);
        s_fail = 1;
      }
    }
  } else {
    // ---- epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 = tile rows,
    // columns 32 h .. 32 h + 31 with h = (w - 2) / 4 ----
    constexpr int EC = OBN / 2;
    const int quad = warp & 3, half = (warp - 2) >> 2;
    const uint32_t trow = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * EC);
    for (int it = 0; it < my_tiles; ++it) {
      if (!mbar_wait(&bars->tfull, it & 1)) {
        if (lane == 0) {
          atomicExch(status, (int)kFlagTimeout);
          s_fail = 1;
        }
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;");
      int m0, n0;
      oz_tile(first_tile + it, tiles_m, tiles_n, m0, n0);
      long long I[EC];
#pragma unroll
      for (int c0 = 0; c0 < EC; c0 += 16) {
        // P_d = acc_d * 2^(7(d-2)) exactly for d <= 6; the tail d = 7..9
        // is summed in FP32 and keeps 3 fraction bits of P_7's unit. Four
        // accumulators at a time keep the register count down.
        uint32_t r[4][16];
#pragma unroll
        for (int a = 0; a < 4; ++a) tmem_ld16_nowait(trow + (uint32_t)(a * OBN + c0), r[a]);
        tmem_ld_wait();
#pragma unroll
        for (int a = 0; a < 4; ++a) touch16(r[a]);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const long long p2 = __float2int_rn(__uint_as_float(r[0][j]));
          const long long p3 = __float2int_rn(__uint_as_float(r[1][j]) * 128.0f);
          const long long p4 = __float2int_rn(__uint_as_float(r[2][j]) * 16384.0f);
          const long long p5 = __float2int_rn(__uint_as_float(r[3][j]) * 2097152.0f);
          I[c0 + j] = (p2 << 38) + (p3 << 31) + (p4 << 24) + (p5 << 17);
        }
#pragma unroll
        for (int a = 0; a < 4; ++a) tmem_ld16_nowait(trow + (uint32_t)((a + 4) * OBN + c0), r[a]);
        tmem_ld_wait();
#pragma unroll
        for (int a = 0; a < 4; ++a) touch16(r[a]);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const long long p6 = __float2int_rn(__uint_as_float(r[0][j]) * 268435456.0f);
          const float tail = (__uint_as_float(r[1][j]) + __uint_as_float(r[2][j])) + __uint_as_float(r[3][j]);
          const long long t8 = __float2ll_rn(tail * 274877906944.0f);  // 2^38
          I[c0 + j] += (p6 << 10) + t8;
        }
      }
      // the accumulators are in registers: the next tile's products may start
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      if (lane == 0) mbar_arrive(&bars->tempty);
      const int row = m0 + quad * 32 + lane;
      if (row < m) {
        const double rsc = alpha * rs[row];
        const int nb0 = n0 + half * EC;
        double* crow = C + (long long)row + (long long)nb0 * ldc;
#pragma unroll
        for (int c0 = 0; c0 < EC; c0 += 8) {
          if (nb0 + c0 >= n) break;
          const int ncol = min(8, n - (nb0 + c0));
          double cv[8], sc[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            cv[j] = (j < ncol) ? crow[(long long)(c0 + j) * ldc] : 0.0;
            sc[j] = (j < ncol) ? __ldg(cs + nb0 + c0 + j) : 0.0;
          }
#pragma unroll
          for (int j = 0; j < 8; ++j)
            if (j < ncol) crow[(long long)(c0 + j) * ldc] = fma(rsc * sc[j], __ll2double_rn(I[c0 + j]), cv[j]);
        }
      }
      if (s_fail) break;
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (s_fail && threadIdx.x == 0) {
    // Drain copies that were issued but never consumed (bounded waits).
    for (int g = s_acons; g < s_aiss; ++g) mbar_wait(&bars->afull[g % A_RING], (g / A_RING) & 1);
    for (int c = s_bcons; c < s_biss; ++c) mbar_wait(&bars->bfull[c & 1], (c >> 1) & 1);
  }
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(OZ_TMEM_COLS));
  }
}

// ---- slicing (integer arithmetic on the FP64 bit patterns) ----------------
//
// With x = +-m 2^q (m the significand as an integer, 53 bits for normal x)
// and a scale exponent e with |x| < 2^e, U = floor(|x| 2^(56-e)) is m shifted
// left by at most 3 bits, or right (dropping the bits below 2^-56 of the
// scale). Slice s (1-based) is bits [56-7s, 63-7s) of U with the sign of x:
// exactly the integer parts of the FP64 truncation x 2^-e = sum a_s 2^-7s.
// With the balancing, A(i,k) is cut against e_i + d_k and B(k,j) against
// f_j - d_k.
constexpr unsigned long long kMagMask = 0x7fffffffffffffffULL;
constexpr unsigned long long kInfBits = 0x7ff0000000000000ULL;

__device__ __forceinline__ unsigned long long oz_fixed(unsigned long long bits, int e) {
  const int bexp = (int)((bits >> 52) & 0x7ff);
  unsigned long long m = bits & 0xfffffffffffffULL;
  int q = -1074;
  if (bexp != 0) {
    m |= 1ULL << 52;
    q = bexp - 1075;
  }
  const int sh = q - e + 56;
  if (sh >= 0) return m << sh;
  if (sh <= -64) return 0ULL;
  return m >> (-sh);
}

// frexp exponent of a magnitude given by its bit pattern (finite, nonzero):
// 2^(ex-1) <= |x| < 2^ex
__device__ __forceinline__ int oz_scale_exp(unsigned long long kmax) {
  const int bexp = (int)(kmax >> 52);
  if (bexp != 0) return bexp - 1022;
  return (63 - __clzll((long long)kmax)) - 1073;  // subnormal
}

// 2^(e - 26) as a double (the epilogue's scale factor half), NaN for a
// non-finite row or column, 0 for a zero one; the caller has checked that
// e - 26 is a normal exponent
__device__ __forceinline__ double oz_scale_value(int e, bool bad) {
  if (bad) return __longlong_as_double(0x7ff8000000000000LL);
  if (e == OZ_NOEXP) return 0.0;
  return __longlong_as_double((long long)((unsigned long long)(e - 26 + 1023) << 52));
}
__device__ __forceinline__ bool oz_scale_in_range(int e) {
  return e == OZ_NOEXP || (e - 26 >= -1022 && e - 26 <= 1023);
}

__device__ __forceinline__ __nv_bfloat16 oz_slice_bf16(unsigned long long U, int s, bool neg) {
  // s is 0-based here: bits [49-7s, 56-7s), weight 2^-7s in the stored slice
  const float a = (float)(unsigned)((U >> (49 - OZ_BITS * s)) & 127ULL);
  return __float2bfloat16_rn((neg ? -a : a) * __int_as_float((127 - OZ_BITS * s) << 23));
}

__device__ __forceinline__ int oz_warp_imax(int v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}
// biased exponent of a finite nonzero value (1 .. 4095), 0 otherwise
__device__ __forceinline__ unsigned oz_ekey(double x) {
  const unsigned long long mag = (unsigned long long)__double_as_longlong(x) & kMagMask;
  return (mag != 0ULL && mag < kInfBits) ? (unsigned)(oz_scale_exp(mag) + OZ_EBIAS) : 0u;
}
// exponent held by a balancing word of this epoch, OZ_NOEXP if none
__device__ __forceinline__ int oz_word_exp(unsigned long long w, unsigned long long epoch) {
  return (w >> 12) == epoch ? (int)(w & 4095ULL) - OZ_EBIAS : OZ_NOEXP;
}

// Balancing exponents of one pass, both operands in one launch. Blocks
// [0, nab): 32 rows of A (m x kb) each; warp w takes columns k = w, w+8, ...
// (one coalesced 256-byte load per column), reduces the lanes' exponent keys
// with one __reduce_max_sync and keeps the column's maximum in shared memory:
// c_k. Blocks after that: 64 columns of B (kb x n) each; warp w takes columns
// w, w+8, ..., lane l rows l, l+32, ...: h_k. Each block publishes its
// maxima with atomicMax into the epoch-tagged words. Small blocks with many
// independent loads, so the pass over both operands runs near copy speed.
__global__ void __launch_bounds__(256)
oz_kscale_kernel(const double* __restrict__ A, long long lda, int m, const double* __restrict__ B,
                 long long ldb, int n, int kb, int nab, unsigned long long* kinfo,
                 unsigned long long epoch) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __shared__ unsigned red[8][OZ_KMAX];
  if ((int)blockIdx.x < nab) {
    const int i = (int)blockIdx.x * 32 + lane;
    const double* arow = A + i;
#pragma unroll 8
    for (int k = warp; k < kb; k += 8) {
      const unsigned v = (i < m) ? oz_ekey(arow[(long long)k * lda]) : 0u;
      const unsigned r = __reduce_max_sync(0xffffffffu, v);
      if (lane == 0) red[0][k] = r;
    }
    __syncthreads();
    const int k = threadIdx.x;
    if (k < kb && red[0][k]) atomicMax(kinfo + OZ_KI_C + k, (epoch << 12) | red[0][k]);
    return;
  }
  const int c0 = ((int)blockIdx.x - nab) * 64;
  unsigned km[OZ_KMAX / 32];
#pragma unroll
  for (int r = 0; r < OZ_KMAX / 32; ++r) km[r] = 0u;
#pragma unroll 2
  for (int q = 0; q < 8; ++q) {
    const int j = c0 + warp + 8 * q;
    if (j < n) {
      const double* col = B + (long long)j * ldb;
#pragma unroll
      for (int r = 0; r < OZ_KMAX / 32; ++r) {
        const int k = lane + 32 * r;
        if (k < kb) km[r] = max(km[r], oz_ekey(col[k]));
      }
    }
  }
#pragma unroll
  for (int r = 0; r < OZ_KMAX / 32; ++r) red[warp][lane + 32 * r] = km[r];
  __syncthreads();
  const int k = threadIdx.x;
  if (k < kb) {
    unsigned v = 0u;
#pragma unroll
    for (int w = 0; w < 8; ++w) v = max(v, red[w][k]);
    if (v) atomicMax(kinfo + OZ_KI_H + k, (epoch << 12) | v);
  }
}

// Both operands in one launch, after oz_kscale_kernel. Blocks [0, m_pad/32):
// 32 rows of A (m x kb, column-major) each, staged through shared memory 64 k
// at a time so that the reads run along the columns; slices Sa[s][i][kk] cut
// against e_i + d_k, and on side A the row's error-budget test. Blocks after
// that: 8 columns of B (kb x n, column-major, a column contiguous in k) each,
// one warp per column; slices Sb[t][j][kk] cut against f_j - d_k, and on side
// B the column's test. Padding rows, columns and k are zero; so is every k
// whose column of A or row of B is zero (its products vanish).
__global__ void __launch_bounds__(256)
oz_split_kernel(const double* __restrict__ A, long long lda, int m, const double* __restrict__ B,
                long long ldb, int n, int kb, int kpad, int m_pad, int n_pad,
                __nv_bfloat16* Sa, __nv_bfloat16* Sb, double* rs, double* cs,
                unsigned long long* kinfo, unsigned long long epoch, int side_b) {
  __shared__ int s_c[OZ_KMAX], s_h[OZ_KMAX], s_d[OZ_KMAX];
  // A blocks: the CTA's 32 rows x kpad of A, as bits, sA[kk * 33 + row],
  // loaded once (before the balancing words, so both reads overlap) and read
  // by the budget test and the slicing
  extern __shared__ unsigned long long sA[];
  const int nrb = m_pad / 32;
  if ((int)blockIdx.x < nrb) {
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = (int)blockIdx.x * 32 + tx;
    unsigned long long v[OZ_KMAX / 8];
#pragma unroll
    for (int q = 0; q < OZ_KMAX / 8; ++q) {
      const int kk = ty + 8 * q;
      v[q] = (i < m && kk < kb) ? (unsigned long long)__double_as_longlong(A[i + (long long)kk * lda])
                                : 0ULL;
    }
#pragma unroll
    for (int q = 0; q < OZ_KMAX / 8; ++q) {
      const int kk = ty + 8 * q;
      if (kk < kpad) sA[kk * 33 + tx] = v[q];
    }
  }
  for (int k = threadIdx.x; k < OZ_KMAX; k += 256) {
    int h = OZ_NOEXP, c = OZ_NOEXP;
    if (k < kb) {
      h = oz_word_exp(kinfo[OZ_KI_H + k], epoch);
      c = oz_word_exp(kinfo[OZ_KI_C + k], epoch);
      if (h == OZ_NOEXP || c == OZ_NOEXP) h = c = OZ_NOEXP;  // k contributes nothing
    }
    s_h[k] = h;
    s_c[k] = c;
    s_d[k] = (c == OZ_NOEXP) ? OZ_NOEXP : (side_b ? -h : c);
  }
  __syncthreads();
  if ((int)blockIdx.x < nrb) {
    __shared__ int redE[8][33], redF[8][33];
    __shared__ int s_e[32];
    __shared__ int s_bad[32];
    __shared__ int s_G;
    const int i0 = blockIdx.x * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int i = i0 + tx;
    if (ty == 0) {  // G = max_k (c_k + h_k)
      int g = OZ_NOEXP;
      for (int q = 0; q < OZ_KMAX / 32; ++q) {
        const int k = tx + 32 * q;
        if (s_c[k] != OZ_NOEXP) g = max(g, s_c[k] + s_h[k]);
      }
      g = oz_warp_imax(g);
      if (tx == 0) s_G = g;
    }
    int em = OZ_NOEXP, fm = OZ_NOEXP, bad = 0;
    if (i < m)
      for (int kk = ty; kk < kb; kk += 8) {
        const unsigned long long mag = sA[kk * 33 + tx] & kMagMask;
        if (mag >= kInfBits) {
          bad = 1;
        } else if (mag != 0ULL && s_d[kk] != OZ_NOEXP) {
          const int ex = oz_scale_exp(mag);
          em = max(em, ex - s_d[kk]);
          fm = max(fm, ex + s_h[kk]);
        }
      }
    redE[ty][tx] = bad ? INT_MAX : em;
    redF[ty][tx] = fm;
    __syncthreads();
    if (ty == 0) {
      int r = OZ_NOEXP, F = OZ_NOEXP;
      bool anybad = false;
      for (int q = 0; q < 8; ++q) {
        anybad |= redE[q][tx] == INT_MAX;
        r = max(r, redE[q][tx] == INT_MAX ? OZ_NOEXP : redE[q][tx]);
        F = max(F, redF[q][tx]);
      }
      s_bad[tx] = anybad ? 1 : 0;
      s_e[tx] = r;
      // side A: row i's bound 2^(e_i + G) against its largest |A||B| term 2^F
      if (!anybad && r != OZ_NOEXP &&
          (!oz_scale_in_range(r) || (!side_b && r + s_G - F > OZ_BUDGET)))
        atomicMax(kinfo + OZ_KI_FLAG, epoch);
      if (i < m_pad) rs[i] = (i < m) ? oz_scale_value(r, anybad) : 0.0;
    }
    __syncthreads();
    const int r = threadIdx.x >> 3, g = threadIdx.x & 7;  // row r, k group g (8 values)
    const int row = i0 + r;
    const int e = s_e[r];
    const bool zero = s_bad[r] != 0 || e == OZ_NOEXP;
    for (int k0 = 0; k0 < kpad; k0 += 64) {
      unsigned long long U[8];
      bool neg[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const int kk = k0 + g * 8 + q;
        const unsigned long long bits = sA[kk * 33 + r];
        neg[q] = (bits >> 63) != 0ULL;
        const int d = s_d[kk];
        U[q] = (zero || d == OZ_NOEXP) ? 0ULL : oz_fixed(bits & kMagMask, e + d);
      }
      if (row < m_pad) {
#pragma unroll
        for (int sl = 0; sl < OZ_S; ++sl) {
          __align__(16) __nv_bfloat16 h[8];
#pragma unroll
          for (int q = 0; q < 8; ++q) h[q] = oz_slice_bf16(U[q], sl, neg[q]);
          *reinterpret_cast<uint4*>(Sa + ((size_t)sl * m_pad + row) * kpad + k0 + g * 8) =
              *reinterpret_cast<const uint4*>(h);
        }
      }
    }
    return;
  }
  // columns of B: one warp per column, lane l holds k = l, l+32, ...
  const int j = ((int)blockIdx.x - nrb) * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (j >= n_pad) return;
  unsigned long long bits[OZ_KMAX / 32];
  int f = OZ_NOEXP, F = OZ_NOEXP, gg = OZ_NOEXP, bad = 0;
#pragma unroll
  for (int q = 0; q < OZ_KMAX / 32; ++q) {
    const int kk = lane + 32 * q;
    bits[q] = (j < n && kk < kb) ? (unsigned long long)__double_as_longlong(B[kk + (long long)j * ldb]) : 0ULL;
    const unsigned long long mag = bits[q] & kMagMask;
    if (s_d[kk] != OZ_NOEXP) gg = max(gg, s_c[kk] + s_h[kk]);
    if (mag >= kInfBits) {
      bad = 1;
    } else if (mag != 0ULL && s_d[kk] != OZ_NOEXP) {
      const int ex = oz_scale_exp(mag);
      f = max(f, ex + s_d[kk]);
      F = max(F, s_c[kk] + ex);
    }
  }
  f = oz_warp_imax(f);
  F = oz_warp_imax(F);
  gg = oz_warp_imax(gg);
  bad = __any_sync(0xffffffffu, bad) ? 1 : 0;
  if (lane == 0) {
    cs[j] = (j < n) ? oz_scale_value(f, bad != 0) : 0.0;
    // side B: column j's bound 2^(f_j + G) against its largest |A||B| term 2^F
    if (j < n && !bad && f != OZ_NOEXP &&
        (!oz_scale_in_range(f) || (side_b && f + gg - F > OZ_BUDGET)))
      atomicMax(kinfo + OZ_KI_FLAG, epoch);
  }
#pragma unroll
  for (int q = 0; q < OZ_KMAX / 32; ++q) {
    const int kk = lane + 32 * q;
    if (kk >= kpad) break;
    const bool neg = (bits[q] >> 63) != 0ULL;
    const int d = s_d[kk];
    const unsigned long long U =
        (bad || f == OZ_NOEXP || d == OZ_NOEXP) ? 0ULL : oz_fixed(bits[q] & kMagMask, f - d);
#pragma unroll
    for (int sl = 0; sl < OZ_S; ++sl) Sb[((size_t)sl * n_pad + j) * kpad + kk] = oz_slice_bf16(U, sl, neg);
  }
}

// 2D map over the slices: rows = S * rows_pad (slice-major), kpad columns of
// BF16, box {64, box_rows}, 128-byte swizzle.
bool make_slice_map(CUtensorMap* map, const void* ptr, int rows_total, int kpad, int box_rows) {
  auto enc = get_encode();
  if (!enc) return false;
  cuuint64_t dims[2] = {(cuuint64_t)kpad, (cuuint64_t)rows_total};
  cuuint64_t strides[1] = {(cuuint64_t)kpad * 2};
  cuuint32_t box[2] = {(cuuint32_t)OBK, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims,
                   strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// dynamic shared memory of oz_split_kernel: the A rows of one CTA
inline size_t oz_split_smem(int kpad) { return (size_t)kpad * 33 * sizeof(unsigned long long); }

cudaError_t oz_smem_once() {
  static const cudaError_t e = cudaFuncSetAttribute(
      ozgemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz_smem_bytes());
  static const cudaError_t e2 = cudaFuncSetAttribute(
      oz_split_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)oz_split_smem(OZ_KMAX));
  return e != cudaSuccess ? e : e2;
}

inline int round_up(int x, int q) { return (x + q - 1) / q * q; }

int g_oz_tiles_per_cta = 4;

}  // namespace

void oz_set_tiles_per_cta(int t) { g_oz_tiles_per_cta = t < 1 ? 1 : (t > 4096 ? 4096 : t); }

size_t oz_scratch_bytes(int m, int n, int k) {
  const size_t kp = (size_t)round_up(k < OZ_KMAX ? k : OZ_KMAX, OBK);
  const size_t mp = (size_t)round_up(m, OBM), np = (size_t)round_up(n, OBN);
  return OZ_KINFO_BYTES + OZ_S * (mp + np) * kp * 2 + (mp + np) * sizeof(double) + 1024;
}

bool oz_fits(const OzScratch& sc, int m, int n, int k) {
  return sc.ptr && oz_scratch_bytes(m, n, k) <= sc.bytes;
}

// Passes that took the FP64 route on the current device since the library
// loaded (the count lives in device memory).
long long oz_fp64_routes() {
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, g_oz_fp64_routes, sizeof(v)) != cudaSuccess) return -1;
  return (long long)v;
}

// Epochs only grow (process-wide, 52 bits: no wrap in practice).
static std::atomic<unsigned long long> g_oz_epochs{0};

unsigned long long oz_new_epoch() {
  return (g_oz_epochs.fetch_add(1) + 1) & ((1ULL << 52) - 1);
}
unsigned long long* oz_ckeys(const OzScratch& sc) {
  return sc.ptr ? reinterpret_cast<unsigned long long*>(sc.ptr) + OZ_KI_C : nullptr;
}
unsigned long long* oz_hkeys(const OzScratch& sc) {
  return sc.ptr ? reinterpret_cast<unsigned long long*>(sc.ptr) + OZ_KI_H : nullptr;
}

// C (m x n) += alpha * A (m x k) * B (k x n), all FP64 column-major, through
// the sliced BF16 product; K is taken in passes of at most 256, each with its
// own balancing, budget test and (when the test trips) FP64 route.
static cudaError_t oz_dgemm_impl(int side_b, unsigned long long keyed_epoch, const OzScratch& sc,
                                 int m, int n, int k, double alpha, const double* A, long long lda,
                                 const double* B, long long ldb, double* C, long long ldc,
                                 int* status, cudaStream_t s, int max_ctas = 0) {
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  if (!oz_fits(sc, m, n, k)) return cudaErrorMemoryAllocation;
  if (keyed_epoch && k > OZ_KMAX) return cudaErrorInvalidValue;
  SL_TRY(oz_smem_once());
  const int m_pad = round_up(m, OBM), n_pad = round_up(n, OBN);
  for (int k0 = 0; k0 < k; k0 += OZ_KMAX) {
    const int kb = (k - k0) < OZ_KMAX ? (k - k0) : OZ_KMAX;
    const int kpad = round_up(kb, OBK);
    const unsigned long long epoch = keyed_epoch ? keyed_epoch : oz_new_epoch();
    unsigned char* p = reinterpret_cast<unsigned char*>(sc.ptr);
    unsigned long long* kinfo = reinterpret_cast<unsigned long long*>(p);
    __nv_bfloat16* sa = reinterpret_cast<__nv_bfloat16*>(p + OZ_KINFO_BYTES);
    __nv_bfloat16* sb = sa + (size_t)OZ_S * m_pad * kpad;
    double* rs = reinterpret_cast<double*>(sb + (size_t)OZ_S * n_pad * kpad);
    double* cs = rs + m_pad;
    const double* Ak = A + (long long)k0 * lda;
    const double* Bk = B + k0;
    const int nab = (m + 31) / 32, nbb = (n + 63) / 64;
    if (!keyed_epoch) {
      oz_kscale_kernel<<<nab + nbb, 256, 0, s>>>(Ak, lda, m, Bk, ldb, n, kb, nab, kinfo, epoch);
      count_launches(1);
    }
    oz_split_kernel<<<m_pad / 32 + n_pad / 8, 256, oz_split_smem(kpad), s>>>(Ak, lda, m, Bk, ldb, n, kb, kpad, m_pad,
                                                          n_pad, sa, sb, rs, cs, kinfo, epoch,
                                                          side_b);
    CUtensorMap ta, tb;
    if (!make_slice_map(&ta, sa, OZ_S * m_pad, kpad, OBM) ||
        !make_slice_map(&tb, sb, OZ_S * n_pad, kpad, OBN))
      return cudaErrorInvalidResourceHandle;
    const int tiles = (m_pad / OBM) * (n_pad / OBN);
    // a few tiles per CTA: enough to overlap one tile's epilogue with the
    // next one's products, few enough that every SM gets work and SMs free
    // up often
    int tpc = std::max(1, std::min(g_oz_tiles_per_cta, tiles / num_sms()));
    if (max_ctas > 0 && (tiles + tpc - 1) / tpc > max_ctas) tpc = (tiles + max_ctas - 1) / max_ctas;
    const int grid = (tiles + tpc - 1) / tpc;
    ozgemm_kernel<<<grid, OZ_THREADS, oz_smem_bytes(), s>>>(ta, tb, m, n, kpad, m_pad, n_pad, rs,
                                                            cs, alpha, C, ldc, tpc, status, Ak,
                                                            lda, Bk, ldb, kb, kinfo, epoch);
    count_launches(2);
    SL_TRY(cudaGetLastError());
  }
  return cudaSuccess;
}

cudaError_t oz_dgemm(const OzScratch& sc, int m, int n, int k, double alpha, const double* A,
                     long long lda, const double* B, long long ldb, double* C, long long ldc,
                     int* status, cudaStream_t s, int max_ctas) {
  return oz_dgemm_impl(0, 0ULL, sc, m, n, k, alpha, A, lda, B, ldb, C, ldc, status, s, max_ctas);
}

cudaError_t oz_dgemm_keyed(const OzScratch& sc, unsigned long long epoch, int m, int n, int k,
                           double alpha, const double* A, long long lda, const double* B,
                           long long ldb, double* C, long long ldc, int* status, cudaStream_t s,
                           int max_ctas) {
  return oz_dgemm_impl(0, epoch, sc, m, n, k, alpha, A, lda, B, ldb, C, ldc, status, s, max_ctas);
}

cudaError_t oz_dgemm_bside(const OzScratch& sc, int m, int n, int k, double alpha,
                           const double* A, long long lda, const double* B, long long ldb,
                           double* C, long long ldc, int* status, cudaStream_t s, int max_ctas) {
  return oz_dgemm_impl(1, 0ULL, sc, m, n, k, alpha, A, lda, B, ldb, C, ldc, status, s, max_ctas);
}

}  // namespace sl
