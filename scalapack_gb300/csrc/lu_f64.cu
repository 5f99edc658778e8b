// FP64 LU factorization and solve on one GB300 (the plain FP64 drop-in path).
//
// Structure follows PDGETRF on a 1x1 grid (SRC/pdgetrf.f:219-295):
//   for each NB-wide block column j:
//     panel      PDGETF2 (SRC/pdgetf2.f:206-237)  -> panel_kernel<double>, blocked by 32
//     swaps      PDLASWP (SRC/pdlaswp.f:163-172)  -> laswp_apply_kernel (composite plan of
//                                                    the panel's interchanges, both sides)
//     U12        PDTRSM  (SRC/pdgetrf.f:280-282)  -> 64x64 block inverses of L11 and
//                                                    sliced products (trsm_strip_kernel
//                                                    in the DMMA mode)
//     update     PDGEMM  (SRC/pdgetrf.f:288-290)  -> oz_dgemm (FP64 from exact BF16 slice
//                                                    products, ozgemm_f64.cu; dgemm DMMA,
//                                                    dgemm_f64.cu, in the DMMA mode)
// with the next panel factored on a second stream (look-ahead), and PDGETRS
// (SRC/pdgetrs.f:250-284): pivots on B (PDLAPIV) as one composed permutation,
// then unit-lower and non-unit-upper blocked solves (diagonal-block inverses
// and sliced products for NOTRAN, substitution strips otherwise).
//
// The NB-wide panel is factored as 32-column sub-panels; each sub-panel is one
// cooperative kernel whose CTAs hold disjoint row slices of the sub-panel in
// shared memory and exchange each column's pivot candidates through tagged
// words in L2 (bounded polls, no grid barrier). The remaining columns of the NB panel are brought up to date
// with the same swap / triangular-solve / GEMM kernels, so the final factors,
// pivots and INFO are those of the reference's column-by-column PDGETF2 in
// exact arithmetic.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "lu_kernels.cuh"
#include "sl_internal.h"

namespace sl {

size_t panel_cand_doubles() { return kPanelCandDoubles; }
static_assert(kPanelCandDoubles == (size_t)PX_WORDS, "exchange area layout");

// Rows per CTA are capped by 200 KB of shared memory (rpc * 33 doubles),
// rounded down to a multiple of 8: 768 rows; one CTA per SM.
int panel_max_rows() { return num_sms() * 768; }
// Global rows of a tall panel: every CTA's slice (rows rounded up to 8).
size_t panel_tile_doubles(int m) {
  return ((size_t)m + (size_t)8 * PMAXG) * PW;
}

static long long g_spin_limit = kSpinLimit;
long long spin_limit() { return g_spin_limit; }
void set_spin_limit(long long polls) { g_spin_limit = polls < 0 ? kSpinLimit : polls; }

static int g_panel_min_rows = 0;  // 0: automatic (FP32 256, FP64 128)
int panel_min_rows() { return g_panel_min_rows; }
static int g_panel_ctas = 64;  // CTAs a panel's rows are spread over (before the minimum rows)
static int g_panel_ib = 2;     // sub-panels per in-panel block (factor_panel)
void set_panel_ib(int ib) { g_panel_ib = ib < 1 ? 1 : (ib > 8 ? 8 : ib); }
int panel_ctas() { return g_panel_ctas; }
void set_panel_ctas(int g) { g_panel_ctas = g < 8 ? 8 : (g > 224 ? 224 : g); }
void set_panel_min_rows(int rows) { g_panel_min_rows = rows <= 0 ? 0 : (rows < 8 ? 8 : (rows > 768 ? 768 : rows)); }

SplitKScratch& splitk_scratch() {
  static SplitKScratch sc;
  return sc;
}

// dst[i] = src[i] + delta (pivot base conversion at the C ABI).
__global__ void ipiv_shift_kernel(const int* __restrict__ src, int* dst, int n, int delta) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i] + delta;
}

cudaError_t ipiv_shift(const int* src, int* dst, int n, int delta, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  ipiv_shift_kernel<<<(n + 255) / 256, 256, 0, s>>>(src, dst, n, delta);
  count_launches(1);
  return cudaGetLastError();
}

// Composed row permutation of the n sequential interchanges j <-> ipiv[j]:
// perm[i] = original row that ends in row i. Thread i walks the interchanges
// backwards from the last, following the row whose content ends in row i
// (interchange j moves it from ipiv[j] to j or from j to ipiv[j]); the pivots
// are compared, never used as addresses, so any IPIV is safe. The walk is the
// same for every thread of a warp (broadcast reads of one pivot at a time),
// from shared memory when n*4 bytes fit in 192 KB.
__global__ void __launch_bounds__(256)
perm_compose_kernel(const int* __restrict__ ipiv, int n, int* perm, int use_smem) {
  extern __shared__ int sp[];
  const int* pv = ipiv;
  if (use_smem) {
    for (int j = threadIdx.x; j < n; j += blockDim.x) sp[j] = ipiv[j];
    __syncthreads();
    pv = sp;
  }
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int q = i;
  for (int j = n - 1; j >= 0; --j) {
    const int p = pv[j];
    q = (q == j) ? p : ((q == p) ? j : q);
  }
  if (i < n) perm[i] = q;
}

cudaError_t perm_compose(const int* dipiv, int n, int* perm, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = sizeof(int) * (size_t)n;
  const int use_smem = smem <= 192 * 1024 ? 1 : 0;
  static const cudaError_t attr = cudaFuncSetAttribute(
      perm_compose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 192 * 1024);
  SL_TRY(attr);
  perm_compose_kernel<<<(n + 255) / 256, 256, use_smem ? smem : 0, s>>>(dipiv, n, perm, use_smem);
  count_launches(1);
  return cudaGetLastError();
}

static int g_f64_update = 1;

void f64_update_set(int mode) { g_f64_update = (mode == 0) ? 0 : 1; }
int f64_update_get() { return g_f64_update; }

// C (m x n) -= A (m x k) * B (k x n) inside the factorization: the sliced
// tensor-core product when selected and its scratch fits, else FP64 DMMA.
// With look-ahead, the update of the columns right of the next panel runs
// beside that panel's kernels (on the auxiliary stream). The panel's
// cooperative kernel makes progress only once all its CTAs are resident, so
// the update keeps at least g_res_min SMs free for it; beyond that it takes
// the SMs it needs to finish within about one panel period (an SM's share of
// the sliced product being g_upd_flops_per_sm in that time) and leaves up to
// g_res_max to the panel chain. (0, 0): the update takes every SM.
static int g_res_min = 24, g_res_max = 88;
// Grid caps in the split step (bit mask): 1 the in-panel products and 2 the
// next panel's update keep to the SMs the trailing update leaves; 4 the
// caller's stream's U12 solve and interchanges keep to the update's SMs.
static int g_cap_mask = 7;
void set_inpanel_cap(int mask) { g_cap_mask = mask & 7; }
static double g_upd_flops_per_sm = 3.2e8;
void set_update_reserve(int min_sms, int max_sms) {
  g_res_min = std::max(0, std::min(min_sms, 120));
  g_res_max = std::max(g_res_min, std::min(max_sms, 120));
}
void set_update_share(double flops_per_sm) {
  g_upd_flops_per_sm = flops_per_sm > 1e6 ? flops_per_sm : 3.2e8;
}
static int update_ctas(double flops) {
  if (g_res_max <= 0) return 0;
  const int S = num_sms();
  const int want = (int)std::ceil(flops / g_upd_flops_per_sm);
  return std::max(1, std::max(S - g_res_max, std::min(S - g_res_min, want)));
}

static cudaError_t lu_update(const OzScratch& sc, int m, int n, int k, double alpha,
                             const double* A, long long lda, const double* B, long long ldb,
                             double* C, long long ldc, const LuWork& ws, cudaStream_t s,
                             int max_ctas = 0) {
  if (g_f64_update == 1 && oz_fits(sc, m, n, k))
    return oz_dgemm(sc, m, n, k, alpha, A, lda, B, ldb, C, ldc, ws.status, s, max_ctas);
  return dgemm(false, m, n, k, alpha, A, lda, B, ldb, 1.0, C, ldc, s);
}

// Inverse of a 64x64 triangular block by column-oriented substitution, all
// columns at once: X = I, then for each pivot row q in solve order, row q of
// X is final (divided by T(q,q) for a non-unit upper T) and every later row
// i loses T(i,q) X(q,:). 256 threads own 16 entries of X each, one shared
// barrier per step: 64 steps instead of a 2000-long dependent chain.
// Ts and X are 64 x 65 shared arrays; returns with X = inv(T).
template <bool LOWER>
__device__ __forceinline__ void tri_inv64_block(double (*Ts)[65], double (*X)[65], double* rd) {
  const int t = threadIdx.x & 63, ib = threadIdx.x >> 6;  // column t, rows ib, ib+4, ...
  if (LOWER) {
    for (int q = 0; q < 63; ++q) {
      const double xq = X[q][t];
      if (t <= q)
        for (int i = q + 1 + ((ib - (q + 1)) & 3); i < 64; i += 4) X[i][t] = fma(-Ts[i][q], xq, X[i][t]);
      __syncthreads();
    }
  } else {
    for (int q = 63; q >= 0; --q) {
      if (threadIdx.x < 64 && t >= q) X[q][t] *= rd[q];
      __syncthreads();
      const double xq = X[q][t];
      if (t >= q)
        for (int i = ib; i < q; i += 4) X[i][t] = fma(-Ts[i][q], xq, X[i][t]);
      __syncthreads();
    }
  }
}

// N_b = inv(L_bb) - I for the 64x64 diagonal blocks of the unit-lower L11
// (jb x jb, leading dimension ldl): block b at Ninv + b*4096, column-major
// with leading dimension 64; a partial last block is padded with the
// identity.
__global__ void __launch_bounds__(256)
unit_lower_inv64_kernel(int jb, const double* __restrict__ L, long long ldl, double* Ninv) {
  extern __shared__ double inv_smem[];  // Ls[64][65] then X[64][65]
  double(*Ls)[65] = reinterpret_cast<double(*)[65]>(inv_smem);
  double(*X)[65] = reinterpret_cast<double(*)[65]>(inv_smem + 64 * 65);
  const int b = blockIdx.x;
  const int r0 = b * 64, rb = min(64, jb - r0);
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    const int r = idx & 63, c = idx >> 6;  // coalesced along rows
    Ls[r][c] = (r < rb && c < r) ? L[(r0 + r) + (long long)(r0 + c) * ldl] : 0.0;
    X[r][c] = (r == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  tri_inv64_block<true>(Ls, X, nullptr);
  double* Nb = Ninv + (size_t)b * 4096;
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    const int i = idx & 63, c = idx >> 6;
    Nb[i + 64 * c] = (i > c) ? X[i][c] : 0.0;
  }
}

// Largest NB whose whole inv(L11) - I is formed at the end of the panel (the
// U12 solve is then one product); larger blocks use 64-row inverses.
constexpr int kFullInvMax = 256;

// X = inv(L) - I for a unit-lower jb x jb L (jb <= 256), one warp per column
// c: x = e_c, then for q = c, c+1, ... x_q is final and every row i > q loses
// L(i,q) x_q -- forward substitution in the order of a strip solve, with x_q
// passed by a shuffle from the lane that owns row q (lane l owns rows l, l+32,
// ..., in registers). Column c costs about (jb-c)^2/2 FMAs on the FP64 pipe,
// so warp pairs take columns p and jb-1-p (equal work per pair) and a CTA of
// kInvColsWarps warps holds kInvColsWarps/2 pairs: the work spreads evenly
// over jb/kInvColsWarps CTAs. L is read from global memory (L2) two columns
// ahead of its use, no shared memory and no block barrier. With a plan to
// make (plan != null), one extra block computes the panel's interchange plan
// (laswp_plan_block) in the same launch: both only read the finished panel.
constexpr int kInvColsWarps = 4;
__host__ __device__ inline int inv_cols_blocks(int jb) {
  const int pairs = (jb + 1) / 2;
  return (pairs + kInvColsWarps / 2 - 1) / (kInvColsWarps / 2);
}
__global__ void __launch_bounds__(32 * kInvColsWarps)
unit_lower_inv_cols_kernel(int jb, const double* __restrict__ L, long long ldl, double* X,
                           int ldx, int k1, int k2, const int* __restrict__ ipiv, int* plan) {
  if (plan != nullptr && (int)blockIdx.x == inv_cols_blocks(jb)) {
    laswp_plan_block(k1, k2, ipiv, plan);
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p = (int)blockIdx.x * (kInvColsWarps / 2) + (warp >> 1);
  const int c = (warp & 1) ? jb - 1 - p : p;
  // the middle column of an odd jb has no partner; pairs past the end none
  if (p >= (jb + 1) / 2 || ((warp & 1) && c == p)) return;
  double xr[8];
#pragma unroll
  for (int t = 0; t < 8; ++t) xr[t] = (lane + 32 * t == c) ? 1.0 : 0.0;
  // L(lane + 32 t, q) for t >= q / 32, rows > q and < jb (0 elsewhere)
  auto load_col = [&](int q, int tq, double* v) {
#pragma unroll
    for (int t = 0; t < 8; ++t) {
      const int i = lane + 32 * t;
      v[t] = (t >= tq && q < jb && i > q && i < jb) ? __ldg(L + i + (long long)q * ldl) : 0.0;
    }
  };
  double v0[8], v1[8];
  load_col(c, c >> 5, v0);
  load_col(c + 1, (c + 1) >> 5, v1);
#pragma unroll
  for (int tq = 0; tq < 8; ++tq) {
    if (32 * tq + 31 < c || 32 * tq >= jb) continue;
    for (int l = (c > 32 * tq ? c - 32 * tq : 0); l < 32; ++l) {
      const int q = 32 * tq + l;
      if (q >= jb) break;
      double v2[8];
      load_col(q + 2, (q + 2) >> 5, v2);  // two columns ahead
      const double xq = __shfl_sync(0xffffffffu, xr[tq], l);
#pragma unroll
      for (int t = tq; t < 8; ++t) xr[t] = fma(-v0[t], xq, xr[t]);
#pragma unroll
      for (int t = 0; t < 8; ++t) {
        v0[t] = v1[t];
        v1[t] = v2[t];
      }
    }
  }
#pragma unroll
  for (int t = 0; t < 8; ++t) {
    const int i = lane + 32 * t;
    if (i < jb) X[i + (long long)c * ldx] = (i > c) ? xr[t] : 0.0;
  }
}

// U12 = L11^-1 A12 (jb x nr, in place). With the sliced product and inverses
// of L11 at hand (formed at the end of its panel): for jb <= 256,
// U12 = A12 + (inv(L11) - I) A12 as one product; otherwise per 64-row block
// b, X_b = A12_b + (inv(L_bb) - I) A12_b, then the rows below lose
// L(below, b) X_b -- every product on the tensor cores, the inverse products
// balanced by the rows of A12, which carry the pivots' scales. Otherwise the
// FP64 strip solve.
static cudaError_t solve_u12(int jb, int nr, const double* L11, long long ldl, double* A12,
                             long long lda, const LuWork& ws, cudaStream_t s, int max_ctas = 0) {
  if (g_f64_update == 1 && ws.dinv64 && jb <= kFullInvMax && oz_fits(ws.oz, jb, nr, jb))
    return oz_dgemm_bside(ws.oz, jb, nr, jb, 1.0, ws.dinv64, jb, A12, lda, A12, lda, ws.status, s,
                          max_ctas);
  if (!(g_f64_update == 1 && ws.dinv64 && jb <= 1024 && oz_fits(ws.oz, jb, nr, 64)))
    return trsm_strip<double, false, false, true>(jb, nr, L11, ldl, A12, lda, s);
  for (int r0 = 0; r0 < jb; r0 += 64) {
    const int w = (jb - r0) < 64 ? (jb - r0) : 64;
    SL_TRY(oz_dgemm_bside(ws.oz, w, nr, w, 1.0, ws.dinv64 + (size_t)(r0 / 64) * 4096, 64,
                          A12 + r0, lda, A12 + r0, lda, ws.status, s));
    if (r0 + w < jb)
      SL_TRY(oz_dgemm(ws.oz, jb - r0 - w, nr, w, -1.0, L11 + (r0 + w) + (long long)r0 * ldl, ldl,
                      A12 + r0, lda, A12 + r0 + w, lda, ws.status, s));
  }
  return cudaSuccess;
}

// PDGETF2 on columns [j, j+jb), rows [j, m): 32-wide cooperative sub-panels,
// each followed by its row interchanges on the rest of the panel, the U solve
// and the GEMM update of the panel's remaining columns.
static cudaError_t factor_panel(int m, double* dA, long long ldda, int* dipiv, int j, int jb,
                                const LuWork& ws, cudaStream_t s) {
  auto Ap = [&](long long i, long long c) { return dA + i + c * ldda; };
  const OzScratch& sc = (ws.aux && s == ws.aux) ? ws.oz_aux : ws.oz;
  phase_begin(kPhPanel, s);
  double pflops = 0.0;
  // Sub-panels are grouped in blocks of g_panel_ib: inside a block only the
  // next sub-panel's columns are brought up to date after each sub-panel
  // (left-looking, with every pivot row of the block so far), and the
  // columns beyond the block once at its end, with the block's rows -- fewer,
  // deeper in-panel products than one per sub-panel over all the remaining
  // columns.
  int blk_r0 = j;  // first row (= column) of the current block
  for (int c = 0, q = 0; c < jb; c += PW, ++q) {
    const int w = (jb - c) < PW ? (jb - c) : PW;
    const int r0 = j + c;
    const int kw = (m - r0) < w ? (m - r0) : w;
    double kflops = 0.0;
    for (int k = 0; k < kw; ++k) kflops += 2.0 * (double)(m - r0 - k - 1) * (w - k - 1) + (m - r0 - k - 1);
    pflops += kflops;
    phase_begin(kPhPanelKernel, s);
    SL_TRY(launch_panel<double>(dA, ldda, m, r0, r0, w, dipiv, ws, s));
    phase_end(kPhPanelKernel, s, kflops, 16.0 * (double)(m - r0) * w);
    phase_begin(kPhPanelUpdate, s);
    SL_TRY(laswp<double>(dA, ldda, r0, r0 + kw, dipiv, j, r0, r0 + w, j + jb, s));
    if (c + w < jb) {
      const bool block_end = (q + 1) % g_panel_ib == 0 || kw < w;
      // columns brought up to date now: the next sub-panel's, or at the end
      // of a block every remaining one; rows: the block's pivot rows (U, by
      // the strip solve) and every row below them (the product)
      const int ncols = block_end ? jb - c - w : ((jb - c - w) < PW ? (jb - c - w) : PW);
      const int kb = r0 + kw - blk_r0;
      const int rl = r0 + kw;  // first row below the block's pivot rows
      // The strip solve also publishes the balancing keys of the product that
      // follows it: the row maxima of its own output (U) and, in extra blocks
      // of the same launch, the column maxima of the block's L.
      const bool keyed = rl < m && g_f64_update == 1 && oz_fits(sc, m - rl, ncols, kb);
      OzKeyJob kj;
      if (keyed) {
        kj.epoch = oz_new_epoch();
        kj.ckeys = oz_ckeys(sc);
        kj.hkeys = oz_hkeys(sc);
        kj.L = Ap(rl, blk_r0);
        kj.ldl = ldda;
        kj.lrows = m - rl;
        kj.lcols = kb;
      }
      SL_TRY((trsm_strip<double, false, false, true>(kb, ncols, Ap(blk_r0, blk_r0), ldda,
                                                      Ap(blk_r0, r0 + w), ldda, s, kj)));
      pflops += (double)kb * kb * ncols;
      if (keyed) {
        SL_TRY(oz_dgemm_keyed(sc, kj.epoch, m - rl, ncols, kb, -1.0, Ap(rl, blk_r0), ldda,
                              Ap(blk_r0, r0 + w), ldda, Ap(rl, r0 + w), ldda, ws.status, s,
                              ws.aux && s == ws.aux ? ws.inpanel_ctas : 0));
        pflops += 2.0 * (double)(m - rl) * ncols * kb;
      } else if (rl < m) {
        SL_TRY(lu_update(sc, m - rl, ncols, kb, -1.0, Ap(rl, blk_r0), ldda, Ap(blk_r0, r0 + w), ldda,
                         Ap(rl, r0 + w), ldda, ws, s));
        pflops += 2.0 * (double)(m - rl) * ncols * kb;
      }
      if (block_end) blk_r0 = r0 + w;
    }
    phase_end(kPhPanelUpdate, s, 0.0, 0.0);
  }
  phase_begin(kPhPanelInverse, s);
  // the panel's interchanges in composite form, for the row interchanges of
  // the other columns (computed here, on the panel's stream)
  const int npiv = (m - j) < jb ? (m - j) : jb;
  const bool want_plan = ws.swap_plan && npiv <= LSW_MAXP;
  // inverses of L11's diagonal blocks for the U12 solve of this step
  if (g_f64_update == 1 && ws.dinv64 && npiv == jb && jb <= kFullInvMax) {
    // inv(L11) - I whole (jb x jb, leading dimension jb), and the interchange
    // plan in the same launch
    if (want_plan && npiv <= 0) SL_TRY(cudaMemsetAsync(ws.swap_plan, 0, sizeof(int), s));
    const bool fused = want_plan && npiv > 0;
    unit_lower_inv_cols_kernel<<<inv_cols_blocks(jb) + (fused ? 1 : 0), 32 * kInvColsWarps, 0, s>>>(
        jb, Ap(j, j), ldda, ws.dinv64, jb, j, j + npiv, dipiv, fused ? ws.swap_plan : nullptr);
    count_launches(1);
    SL_TRY(cudaGetLastError());
  } else if (want_plan) {
    SL_TRY(laswp_plan(j, j + npiv, dipiv, ws.swap_plan, s));
  }
  if (g_f64_update == 1 && ws.dinv64 && npiv == jb && jb > kFullInvMax && jb <= 1024) {
    constexpr int kInvSmem = 2 * 64 * 65 * (int)sizeof(double);
    static const cudaError_t attr = cudaFuncSetAttribute(
        unit_lower_inv64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kInvSmem);
    SL_TRY(attr);
    unit_lower_inv64_kernel<<<(jb + 63) / 64, 256, kInvSmem, s>>>(jb, Ap(j, j), ldda, ws.dinv64);
    count_launches(1);
  }
  phase_end(kPhPanelInverse, s, (double)jb * jb * jb / 3.0, 16.0 * (double)jb * jb);
  phase_end(kPhPanel, s, pflops, 16.0 * (double)(m - j) * jb);
  return cudaSuccess;
}

// Step 0 of the right-looking loop while the columns arrive in chunks (see
// dgetrf_device; m, n > 2 nb, panel 0 factored): the next panel's columns
// first, then the look-ahead panel on ws.aux, then the remaining columns of
// each chunk once it has landed.
template <typename WaitCols>
static cudaError_t step0_by_chunks(int m, int n, double* dA, long long ldda, int* dipiv, int nb,
                                   const LuWork& ws, cudaStream_t s, WaitCols& wait_cols) {
  auto Ap = [&](long long i, long long c) { return dA + i + c * ldda; };
  const int mn = m < n ? m : n;
  const int jb = nb, jn = nb;
  const int jb2 = (mn - jn) < nb ? (mn - jn) : nb;
  // step 0 on columns [c0, c1): interchanges, U12 solve, trailing update
  auto step_cols = [&](int c0, int c1, bool planned, const LuWork& w) -> cudaError_t {
    if (c1 <= c0) return cudaSuccess;
    const int nc = c1 - c0;
    phase_begin(kPhLaswp, s);
    if (planned) SL_TRY(laswp_planned<double>(dA, ldda, 0, jb, dipiv, w.swap_plan, 0, 0, c0, c1, s));
    else SL_TRY(laswp<double>(dA, ldda, 0, jb, dipiv, 0, 0, c0, c1, s));
    phase_end(kPhLaswp, s, 0.0, 32.0 * jb * (double)nc);
    phase_begin(kPhTrsm, s);
    SL_TRY(solve_u12(jb, nc, Ap(0, 0), ldda, Ap(0, c0), ldda, w, s));
    phase_end(kPhTrsm, s, (double)jb * jb * nc, 8.0 * (0.5 * jb * jb + 2.0 * jb * nc));
    if (jn < m) {
      const double mr = (double)(m - jn);
      phase_begin(kPhGemm, s);
      SL_TRY(lu_update(w.oz, m - jn, nc, jb, -1.0, Ap(jn, 0), ldda, Ap(0, c0), ldda, Ap(jn, c0),
                       ldda, w, s));
      phase_end(kPhGemm, s, 2.0 * mr * nc * jb, 8.0 * (mr * jb + (double)jb * nc + 2.0 * mr * nc));
    }
    return cudaSuccess;
  };
  SL_TRY(wait_cols(jn + jb2));
  SL_TRY(step_cols(jn, jn + jb2, true, ws));
  // the look-ahead panel rewrites the interchange plan and ws.dinv64: the
  // rest of step 0 reads dipiv and a copy of panel 0's inverses instead
  LuWork w0 = ws;
  w0.swap_plan = nullptr;
  if (g_f64_update == 1 && ws.dinv64) {
    SL_TRY(cudaMemcpyAsync(ws.dinv64_step0, ws.dinv64,
                           (jb <= kFullInvMax ? (size_t)jb * jb : (size_t)((jb + 63) / 64) * 4096) * sizeof(double),
                           cudaMemcpyDeviceToDevice, s));
    w0.dinv64 = ws.dinv64_step0;
  }
  SL_TRY(cudaEventRecord(ws.ev_next, s));
  SL_TRY(cudaStreamWaitEvent(ws.aux, ws.ev_next, 0));
  SL_TRY(factor_panel(m, dA, ldda, dipiv, jn, jb2, ws, ws.aux));
  SL_TRY(cudaEventRecord(ws.ev_panel, ws.aux));
  const int nck = ws.ncol_chunks < kMaxColChunks ? ws.ncol_chunks : kMaxColChunks;
  for (int c = 0; c < nck; ++c) {
    const int lo = c ? ws.col_end[c - 1] : 0, hi = ws.col_end[c];
    const int a = lo > jn + jb2 ? lo : jn + jb2, b = hi < n ? hi : n;
    if (b <= a) continue;
    SL_TRY(wait_cols(b));
    SL_TRY(step_cols(a, b, false, w0));
  }
  return wait_cols(INT_MAX);
}

// Right-looking blocked LU. With look-ahead resources in `ws`, the panel of
// step j+1 is factored on ws.aux while the trailing update of step j runs on
// s: the columns of the next panel are updated first (event ev_next), the
// next panel starts as soon as they are ready, and step j+1 waits for it
// (event ev_panel). Panel and update touch disjoint columns, and each element
// is accumulated in the same order either way, so the factors are the same.
//
// With columns still arriving (ws.ncol_chunks > 0), s waits for each column
// chunk just before the first operation on it: panel 0 starts when its
// columns are in place, and step 0's interchanges, U12 solve and update run
// chunk by chunk as the rest lands. The interchanges and the update are
// independent per column; the U12 solve's first product balances its slices
// by the row maxima of the columns it is given, so those rows agree with the
// whole-width step to rounding (same pivots). After the look-ahead panel is
// launched the step-0 operations must not
// read the per-panel scratch that panel overwrites (the interchange plan and
// L11's block inverses): they take the interchanges from dipiv and a copy of
// the inverses (ws.dinv64_step0).
cudaError_t dgetrf_device(int m, int n, double* dA, long long ldda, int* dipiv, int nb,
                          const LuWork& ws, cudaStream_t s) {
  SL_TRY(cudaMemsetAsync(ws.status, 0, sizeof(int), s));
  SL_TRY(cudaMemsetAsync(ws.info_col, 0x7f, sizeof(int), s));
  const int mn = m < n ? m : n;
  if (nb > 1024) nb = 1024;
  auto Ap = [&](long long i, long long j) { return dA + i + j * ldda; };
  const bool lookahead = ws.aux && ws.ev_next && ws.ev_panel && mn > 2 * nb;
  // column chunks: s waits for every chunk that starts below column `upto`
  const int nck = (ws.ncol_chunks > 0 && ws.col_end && ws.ev_cols)
                      ? (ws.ncol_chunks < kMaxColChunks ? ws.ncol_chunks : kMaxColChunks) : 0;
  int next_chunk = 0;
  auto wait_cols = [&](int upto) -> cudaError_t {
    while (next_chunk < nck && (next_chunk ? ws.col_end[next_chunk - 1] : 0) < upto) {
      SL_TRY(cudaStreamWaitEvent(s, ws.ev_cols[next_chunk], 0));
      ++next_chunk;
    }
    return cudaSuccess;
  };
  const bool stream_step0 = nck > 0 && lookahead && ws.dinv64_step0 && ws.col_end[nck - 1] >= n;
  SL_TRY(wait_cols(stream_step0 ? nb : INT_MAX));
  if (mn > 0) SL_TRY(factor_panel(m, dA, ldda, dipiv, 0, (mn < nb ? mn : nb), ws, s));
  bool panel_on_aux = false;
  if (stream_step0) {
    SL_TRY(step0_by_chunks(m, n, dA, ldda, dipiv, nb, ws, s, wait_cols));
    panel_on_aux = true;
  }
  // Split look-ahead step (both buffer sets present, the panel stream's
  // scratch holding an m x nb x nb product): once panel j is factored, the
  // panel stream brings the next panel's columns up to date itself (their
  // interchanges, U12 solve and update) and factors that panel, while the
  // caller's stream handles every other column -- so only the next panel's
  // share of the step lies between two panels. cur holds the inverse and
  // interchange plan of the panel just factored, nxt receives the next one's;
  // the caller's stream is done with cur's before the panel stream rewrites
  // them two panels later (it waits for ev_next, recorded after that work).
  LuWork cur = ws, nxt = ws;
  const bool split = lookahead && ws.dinv64_alt && ws.swap_plan_alt && g_f64_update == 1 &&
                     oz_fits(ws.oz_aux, m, nb, nb);
  if (split) {
    nxt.dinv64 = ws.dinv64_alt;
    nxt.swap_plan = ws.swap_plan_alt;
  }
  for (int j = stream_step0 ? nb : 0; j < mn; j += nb) {
    const int jb = (mn - j) < nb ? (mn - j) : nb;
    if (panel_on_aux) SL_TRY(cudaStreamWaitEvent(s, ws.ev_panel, 0));
    panel_on_aux = false;
    const int jn = j + jb;                                   // next panel's first column
    const int jb2 = jn < mn ? ((mn - jn) < nb ? (mn - jn) : nb) : 0;
    if (split && jb2 > 0) {
      const double mr = (double)(m - jn);
      // panel j, and every update of the caller's stream before it
      SL_TRY(cudaEventRecord(ws.ev_next, s));
      SL_TRY(cudaStreamWaitEvent(ws.aux, ws.ev_next, 0));
      LuWork aw = cur;
      aw.oz = ws.oz_aux;
      phase_begin(kPhLaswp, ws.aux);
      SL_TRY(laswp_planned<double>(dA, ldda, j, jn, dipiv, cur.swap_plan, jn, jn + jb2, jn + jb2, jn + jb2, ws.aux));
      phase_end(kPhLaswp, ws.aux, 0.0, 32.0 * jb * (double)jb2);
      phase_begin(kPhTrsm, ws.aux);
      SL_TRY(solve_u12(jb, jb2, Ap(j, j), ldda, Ap(j, jn), ldda, aw, ws.aux));
      phase_end(kPhTrsm, ws.aux, (double)jb * jb * jb2, 8.0 * (0.5 * jb * jb + 2.0 * jb * jb2));
      // the next panel's update and in-panel products run on the SMs the
      // update of the other columns (beside them) leaves
      const int rest_cols = n - jn - jb2;
      const int upd = rest_cols > 0 ? update_ctas(2.0 * mr * rest_cols * jb) : 0;
      const int free_sms = upd > 0 ? num_sms() - upd : 0;
      phase_begin(kPhGemm, ws.aux);
      SL_TRY(lu_update(ws.oz_aux, m - jn, jb2, jb, -1.0, Ap(jn, j), ldda, Ap(j, jn), ldda, Ap(jn, jn),
                       ldda, ws, ws.aux, (g_cap_mask & 2) ? free_sms : 0));
      phase_end(kPhGemm, ws.aux, 2.0 * mr * jb2 * jb, 8.0 * (mr * jb + (double)jb * jb2 + 2.0 * mr * jb2));
      nxt.inpanel_ctas = (g_cap_mask & 1) ? free_sms : 0;
      SL_TRY(factor_panel(m, dA, ldda, dipiv, jn, jb2, nxt, ws.aux));
      SL_TRY(cudaEventRecord(ws.ev_panel, ws.aux));
      panel_on_aux = true;
      // the other columns on the caller's stream
      const int c2 = jn + jb2, rest = n - c2;
      const int main_cap = (g_cap_mask & 4) ? upd : 0;
      phase_begin(kPhLaswp, s);
      SL_TRY(laswp_planned<double>(dA, ldda, j, jn, dipiv, cur.swap_plan, 0, j, c2, n, s, main_cap));
      phase_end(kPhLaswp, s, 0.0, 32.0 * jb * (double)(n - jb - jb2));
      if (rest > 0) {
        phase_begin(kPhTrsm, s);
        SL_TRY(solve_u12(jb, rest, Ap(j, j), ldda, Ap(j, c2), ldda, cur, s, main_cap));
        phase_end(kPhTrsm, s, (double)jb * jb * rest, 8.0 * (0.5 * jb * jb + 2.0 * jb * rest));
        phase_begin(kPhGemm, s);
        SL_TRY(lu_update(ws.oz, m - jn, rest, jb, -1.0, Ap(jn, j), ldda, Ap(j, c2), ldda, Ap(jn, c2),
                         ldda, ws, s, update_ctas(2.0 * mr * rest * jb)));
        phase_end(kPhGemm, s, 2.0 * mr * rest * jb, 8.0 * (mr * jb + (double)jb * rest + 2.0 * mr * rest));
      }
      std::swap(cur, nxt);
      continue;
    }
    // ---- PDLASWP on the left and right column blocks ----
    phase_begin(kPhLaswp, s);
    SL_TRY(laswp_planned<double>(dA, ldda, j, j + jb, dipiv, cur.swap_plan, 0, j, j + jb, n, s));
    phase_end(kPhLaswp, s, 0.0, 32.0 * jb * (double)(n - jb));
    if (jn < n) {
      // ---- PDTRSM: U12 = L11^{-1} A12 ----
      const double nr = (double)(n - jn);
      phase_begin(kPhTrsm, s);
      SL_TRY(solve_u12(jb, n - jn, Ap(j, j), ldda, Ap(j, jn), ldda, cur, s));
      phase_end(kPhTrsm, s, (double)jb * jb * nr, 8.0 * (0.5 * jb * jb + 2.0 * jb * nr));
      // ---- PDGEMM: A22 -= L21 * U12 ----
      if (jn < m) {
        const double mr = (double)(m - jn);
        if (lookahead && jb2 > 0) {
          // next panel's columns first, then the panel on the look-ahead stream
          phase_begin(kPhGemm, s);
          SL_TRY(lu_update(ws.oz, m - jn, jb2, jb, -1.0, Ap(jn, j), ldda, Ap(j, jn), ldda,
                           Ap(jn, jn), ldda, ws, s));
          phase_end(kPhGemm, s, 2.0 * mr * jb2 * jb, 8.0 * (mr * jb + (double)jb * jb2 + 2.0 * mr * jb2));
          SL_TRY(cudaEventRecord(ws.ev_next, s));
          SL_TRY(cudaStreamWaitEvent(ws.aux, ws.ev_next, 0));
          SL_TRY(factor_panel(m, dA, ldda, dipiv, jn, jb2, ws, ws.aux));
          SL_TRY(cudaEventRecord(ws.ev_panel, ws.aux));
          panel_on_aux = true;
          const int rest = n - jn - jb2;
          if (rest > 0) {
            phase_begin(kPhGemm, s);
            SL_TRY(lu_update(ws.oz, m - jn, rest, jb, -1.0, Ap(jn, j), ldda, Ap(j, jn + jb2), ldda,
                             Ap(jn, jn + jb2), ldda, ws, s,
                             update_ctas(2.0 * mr * rest * jb)));
            phase_end(kPhGemm, s, 2.0 * mr * rest * jb, 8.0 * (mr * jb + (double)jb * rest + 2.0 * mr * rest));
          }
        } else {
          phase_begin(kPhGemm, s);
          SL_TRY(lu_update(ws.oz, m - jn, n - jn, jb, -1.0, Ap(jn, j), ldda, Ap(j, jn), ldda,
                           Ap(jn, jn), ldda, ws, s));
          phase_end(kPhGemm, s, 2.0 * mr * nr * jb, 8.0 * (mr * jb + jb * nr + 2.0 * mr * nr));
        }
      }
    }
    if (jb2 > 0 && !panel_on_aux) SL_TRY(factor_panel(m, dA, ldda, dipiv, jn, jb2, ws, s));
  }
  if (panel_on_aux) SL_TRY(cudaStreamWaitEvent(s, ws.ev_panel, 0));
  return cudaGetLastError();
}

// Off-diagonal update of the blocked solves: C += alpha op(A) B.
template <>
cudaError_t gemm_update<double>(bool transa, int m, int n, int k, double alpha, const double* A,
                                long long lda, const double* B, long long ldb, double* C,
                                long long ldc, cudaStream_t s) {
  if (n <= 16) return gemm_skinny<double>(transa, m, n, k, alpha, A, lda, B, ldb, C, ldc, s);
  return dgemm(transa, m, n, k, alpha, A, lda, B, ldb, 1.0, C, ldc, s);
}

// Inverses of the 64x64 diagonal blocks of the unit-lower L (LOWER) or the
// non-unit upper U of an n x n LU factor, for the blocked solves: block b at
// D + b*4096, column-major with leading dimension 64 (D[c*64 + r] =
// inv(T_bb)(r, c)); a partial last block is padded with the identity.
template <bool LOWER>
__global__ void __launch_bounds__(256)
tri_inv64_kernel(int n, const double* __restrict__ A, long long lda, double* D) {
  extern __shared__ double inv_smem[];  // Ts[64][65], X[64][65], rdiag[64]
  double(*Ts)[65] = reinterpret_cast<double(*)[65]>(inv_smem);
  double(*X)[65] = reinterpret_cast<double(*)[65]>(inv_smem + 64 * 65);
  double* rd = inv_smem + 2 * 64 * 65;
  const int b = blockIdx.x;
  const int r0 = b * 64, rb = min(64, n - r0);
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    const int r = idx & 63, c = idx >> 6;
    double v = 0.0;
    if (r < rb && c < rb && (LOWER ? c < r : c >= r)) v = A[(r0 + r) + (long long)(r0 + c) * lda];
    Ts[r][c] = v;
    X[r][c] = (r == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  if (!LOWER && threadIdx.x < 64) rd[threadIdx.x] = (threadIdx.x < rb) ? 1.0 / Ts[threadIdx.x][threadIdx.x] : 1.0;
  __syncthreads();
  tri_inv64_block<LOWER>(Ts, X, rd);
  double* Db = D + (size_t)b * 4096;
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    const int r = idx & 63, c = idx >> 6;
    Db[c * 64 + r] = X[r][c];
  }
}

// Balancing keys of the blocked NOTRAN solve's sliced products, once per
// solve: for column k of the factor, with b = k / 128, ck[k] is the largest
// exponent key of the unit-lower L's entries in rows [(b+1)*128, n) and
// ck[npad + k] that of U's entries in rows [0, b*128) -- the rows of the A
// operand of the product that follows block b's solve (the low 12 bits of
// oz_key_word; 0: no finite nonzero entry). One warp per column.
__global__ void __launch_bounds__(256)
solve_ckeys_kernel(int n, const double* __restrict__ A, long long lda, unsigned* ck, int npad) {
  const int k = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (k >= n) return;
  const double* col = A + (long long)k * lda;
  const int lo = (k / 128) * 128, hi = lo + 128;
  unsigned kl = 0u, ku = 0u;
  for (int i = hi + lane; i < n; i += 32) kl = max(kl, (unsigned)oz_key_word(col[i], 0ULL));
  for (int i = lane; i < lo; i += 32) ku = max(ku, (unsigned)oz_key_word(col[i], 0ULL));
  kl = __reduce_max_sync(0xffffffffu, kl);
  ku = __reduce_max_sync(0xffffffffu, ku);
  if (lane == 0) {
    ck[k] = kl;
    ck[npad + k] = ku;
  }
}

// One block step of the blocked NOTRAN solve: X(k0:k0+kb, c) =
// inv(T_bb) X(k0:k0+kb, c) for the 128-row block at k0 of the unit-lower L
// (LOWER, forward) or the upper U (backward), from the inverses of its two
// 64x64 diagonal blocks and its off-diagonal 64x64 block, staged in shared
// memory. CTA c < nrhs takes right-hand side c (threads 0..127 one row each);
// with ckeys set, the CTAs also publish the balancing keys of the sliced
// product that follows (A: the factor's columns k0..k0+kb outside the block,
// B: the solved rows): the h keys from each column's solved values and, in
// the extra CTA nrhs, the c keys from ck.
constexpr int kBlkSmem = 3 * 64 * 64 * (int)sizeof(double);
template <bool LOWER>
__global__ void __launch_bounds__(256)
solve_block128_kernel(int kb, const double* __restrict__ A, long long lda, int k0,
                      const double* __restrict__ D, double* X, long long ldx, int nrhs,
                      const unsigned* __restrict__ ck, unsigned long long* ckeys,
                      unsigned long long* hkeys, unsigned long long epoch) {
  extern __shared__ double blk_smem[];  // D0, D1 and the off-diagonal block O, each [c*64 + r]
  __shared__ double xs[128], ys[128];
  const int c = blockIdx.x, t = threadIdx.x;
  if (c == nrhs) {  // the c keys of the following product
    if (t < kb && ck[k0 + t]) atomicMax(ckeys + t, (epoch << 12) | ck[k0 + t]);
    return;
  }
  double* x = X + k0 + (long long)c * ldx;
  const int b0 = k0 / 64;  // first 64-block
  const int w0 = kb < 64 ? kb : 64, w1 = kb - w0;
  double* D0s = blk_smem;
  double* D1s = blk_smem + 4096;
  double* Os = blk_smem + 2 * 4096;
  {
    // every load of the staging is issued before the first store (one
    // memory round trip): D0 and D1 (D1 follows D0 in memory; only when the
    // block has a second half), O = L10 (rows 64.., columns 0..) or U01
    // (rows 0.., columns 64..), [i*64 + r], and this column's right-hand side
    const double2* Dg = reinterpret_cast<const double2*>(D + (size_t)b0 * 4096);
    const int nd = (w1 > 0 ? 2 : 1) * 2048;
    const double xv = (t < kb) ? x[t] : 0.0;
    double2 rd[16];
    double ro[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int idx = t + 256 * q;
      rd[q] = idx < nd ? Dg[idx] : make_double2(0.0, 0.0);
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int idx = t + 256 * q;
      const int r = idx & 63, i = idx >> 6;
      const bool in = LOWER ? (r < w1 && i < w0) : (r < w0 && i < w1);
      const long long off = LOWER ? (k0 + 64 + r) + (long long)(k0 + i) * lda
                                  : (k0 + r) + (long long)(k0 + 64 + i) * lda;
      ro[q] = in ? A[off] : 0.0;
    }
    double2* d = reinterpret_cast<double2*>(blk_smem);
#pragma unroll
    for (int q = 0; q < 16; ++q) d[t + 256 * q] = rd[q];
#pragma unroll
    for (int q = 0; q < 16; ++q) Os[t + 256 * q] = ro[q];
    if (t < 128) xs[t] = xv;
  }
  __syncthreads();
  if (LOWER) {
    // y0 = inv(L00) x0; x1 -= L10 y0; y1 = inv(L11) x1
    if (t < 64) {
      double acc = 0.0;
      for (int i = 0; i < 64; ++i) acc = fma(D0s[i * 64 + t], xs[i], acc);
      ys[t] = acc;
    }
    __syncthreads();
    if (t >= 64 && t < 128 && t - 64 < w1) {
      double acc = xs[t];
      for (int i = 0; i < w0; ++i) acc = fma(-Os[i * 64 + (t - 64)], ys[i], acc);
      xs[t] = acc;
    }
    __syncthreads();
    if (t >= 64 && t < 128 && w1 > 0) {  // (no second 64-block when kb <= 64)
      const int r = t - 64;
      double acc = 0.0;
      for (int i = 0; i < 64; ++i) acc = fma(D1s[i * 64 + r], xs[64 + i], acc);
      ys[t] = acc;
    }
  } else {
    // y1 = inv(U11) x1; x0 -= U01 y1; y0 = inv(U00) x0
    if (t >= 64 && t < 128 && w1 > 0) {
      const int r = t - 64;
      double acc = 0.0;
      for (int i = 0; i < 64; ++i) acc = fma(D1s[i * 64 + r], xs[64 + i], acc);
      ys[t] = acc;
    } else if (t >= 64 && t < 128) {
      ys[t] = 0.0;
    }
    __syncthreads();
    if (t < 64 && w1 > 0) {
      double acc = xs[t];
      for (int i = 0; i < w1; ++i) acc = fma(-Os[i * 64 + t], ys[64 + i], acc);
      xs[t] = acc;
    }
    __syncthreads();
    if (t < 64) {
      double acc = 0.0;
      for (int i = 0; i < 64; ++i) acc = fma(D0s[i * 64 + t], xs[i], acc);
      ys[t] = acc;
    }
  }
  __syncthreads();
  if (t < kb) {
    x[t] = ys[t];
    if (hkeys) {
      const unsigned long long w = oz_key_word(ys[t], epoch);
      if (w) atomicMax(hkeys + t, w);
    }
  }
}

// Blocked NOTRAN solve with the diagonal-block inverses (ws.dinv_solve: L
// blocks, then U blocks, then the column keys) and the off-diagonal updates
// as sliced products on the tensor cores: 128-row blocks, each applied by
// inverse and then subtracted from the rest. The products take their
// balancing keys from the block step (no key pass over the factor per step).
static cudaError_t tri_solve_inv(bool lower, int n, int nrhs, const double* A, long long lda,
                                 double* X, long long ldx, const LuWork& ws, cudaStream_t s) {
  constexpr int KB = 128;
  const int nblk = (n + KB - 1) / KB;
  const int nb64 = (n + 63) / 64;
  const double* D = ws.dinv_solve + (lower ? 0 : (size_t)nb64 * 4096);
  const unsigned* ck = reinterpret_cast<const unsigned*>(ws.dinv_solve + (size_t)2 * nb64 * 4096) +
                       (lower ? 0 : nb64 * 64);
  unsigned long long* ckeys = oz_ckeys(ws.oz);
  unsigned long long* hkeys = oz_hkeys(ws.oz);
  for (int bi = 0; bi < nblk; ++bi) {
    const int b = lower ? bi : nblk - 1 - bi;
    const int k0 = b * KB, kb = (n - k0) < KB ? (n - k0) : KB;
    const int rest = lower ? n - k0 - kb : k0;
    const unsigned long long ep = rest > 0 ? oz_new_epoch() : 0ULL;
    if (lower)
      solve_block128_kernel<true><<<nrhs + (rest > 0 ? 1 : 0), 256, kBlkSmem, s>>>(
          kb, A, lda, k0, D, X, ldx, nrhs, ck, ckeys, rest > 0 ? hkeys : nullptr, ep);
    else
      solve_block128_kernel<false><<<nrhs + (rest > 0 ? 1 : 0), 256, kBlkSmem, s>>>(
          kb, A, lda, k0, D, X, ldx, nrhs, ck, ckeys, rest > 0 ? hkeys : nullptr, ep);
    count_launches(1);
    SL_TRY(cudaGetLastError());
    if (rest > 0 && lower)
      SL_TRY(oz_dgemm_keyed(ws.oz, ep, rest, nrhs, kb, -1.0, A + (k0 + kb) + (long long)k0 * lda, lda,
                            X + k0, ldx, X + k0 + kb, ldx, ws.status, s));
    else if (rest > 0)
      SL_TRY(oz_dgemm_keyed(ws.oz, ep, k0, nrhs, kb, -1.0, A + (long long)k0 * lda, lda, X + k0, ldx,
                            X, ldx, ws.status, s));
  }
  return cudaSuccess;
}

cudaError_t dgetrs_device(char trans, int n, int nrhs, const double* dA, long long ldda,
                          const int* dipiv, double* dB, long long lddb, const LuWork& ws,
                          cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return cudaSuccess;
  const bool notran = (trans == 'N' || trans == 'n');
  phase_begin(kPhSolve, s);
  SL_TRY(perm_compose(dipiv, n, ws.perm, s));
  double* X = ws.bswap;  // n x nrhs, ld = n
  // any NRHS whose products fit the scratch (PDGETRI solves with NRHS = N)
  const bool inv_path = g_f64_update == 1 && ws.dinv_solve && ws.dinv_solve_len >= kSolveInvDoubles(n) &&
                        oz_fits(ws.oz, n, nrhs, 128);
  if (notran && inv_path) {
    SL_TRY((permute_rows<double, double>(dB, lddb, X, n, ws.perm, n, nrhs, 0, s)));
    const int nb64 = (n + 63) / 64;
    constexpr int kInvSmem = (2 * 64 * 65 + 64) * (int)sizeof(double);
    static const cudaError_t a0 = cudaFuncSetAttribute(
        tri_inv64_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kInvSmem);
    static const cudaError_t a1 = cudaFuncSetAttribute(
        tri_inv64_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kInvSmem);
    static const cudaError_t a2 = cudaFuncSetAttribute(
        solve_block128_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBlkSmem);
    static const cudaError_t a3 = cudaFuncSetAttribute(
        solve_block128_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kBlkSmem);
    SL_TRY(a0);
    SL_TRY(a1);
    SL_TRY(a2);
    SL_TRY(a3);
    tri_inv64_kernel<true><<<nb64, 256, kInvSmem, s>>>(n, dA, ldda, ws.dinv_solve);
    tri_inv64_kernel<false><<<nb64, 256, kInvSmem, s>>>(n, dA, ldda, ws.dinv_solve + (size_t)nb64 * 4096);
    solve_ckeys_kernel<<<(n + 7) / 8, 256, 0, s>>>(
        n, dA, ldda, reinterpret_cast<unsigned*>(ws.dinv_solve + (size_t)2 * nb64 * 4096), nb64 * 64);
    count_launches(3);
    SL_TRY(cudaGetLastError());
    SL_TRY(tri_solve_inv(true, n, nrhs, dA, ldda, X, n, ws, s));
    SL_TRY(tri_solve_inv(false, n, nrhs, dA, ldda, X, n, ws, s));
    SL_TRY(cudaMemcpy2DAsync(dB, lddb * sizeof(double), X, n * sizeof(double),
                             n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s));
  } else if (notran) {
    SL_TRY((permute_rows<double, double>(dB, lddb, X, n, ws.perm, n, nrhs, 0, s)));
    SL_TRY(tri_solve<double>(true, false, true, n, nrhs, dA, ldda, X, n, s));
    SL_TRY(tri_solve<double>(false, false, false, n, nrhs, dA, ldda, X, n, s));
    SL_TRY(cudaMemcpy2DAsync(dB, lddb * sizeof(double), X, n * sizeof(double),
                             n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s));
  } else {
    SL_TRY(cudaMemcpy2DAsync(X, n * sizeof(double), dB, lddb * sizeof(double),
                             n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s));
    SL_TRY(tri_solve<double>(false, true, false, n, nrhs, dA, ldda, X, n, s));
    SL_TRY(tri_solve<double>(true, true, true, n, nrhs, dA, ldda, X, n, s));
    SL_TRY((permute_rows<double, double>(X, n, dB, lddb, ws.perm, n, nrhs, 1, s)));
  }
  phase_end(kPhSolve, s, 2.0 * (double)n * n * nrhs, 8.0 * ((double)n * n + 4.0 * (double)n * nrhs));
  return cudaSuccess;
}

}  // namespace sl
