// FP64 LU factorization and solve on one GB300 (the plain FP64 drop-in path).
//
// Structure follows PDGETRF on a 1x1 grid (SRC/pdgetrf.f:219-295):
//   for each NB-wide block column j:
//     panel      PDGETF2 (SRC/pdgetf2.f:206-237)  -> panel_f64_kernel, blocked by 32
//     swaps      PDLASWP (SRC/pdlaswp.f:163-172)  -> laswp_kernel (left and right parts)
//     U12        PDTRSM  (SRC/pdgetrf.f:280-282)  -> trsm_strip_kernel
//     update     PDGEMM  (SRC/pdgetrf.f:288-290)  -> dgemm (DMMA, dgemm_f64.cu)
// and PDGETRS (SRC/pdgetrs.f:250-284): pivots on B (PDLAPIV), unit-lower and
// non-unit-upper solves (blocked by 64, diagonal strip + narrow update).
//
// The NB-wide panel is factored as 32-column sub-panels; each sub-panel is one
// cooperative kernel whose CTAs hold disjoint row slices of the sub-panel in
// shared memory and meet at one bounded grid barrier per column (pivot search
// across CTAs). The remaining columns of the NB panel are brought up to date
// with the same swap / triangular-solve / GEMM kernels, so the final factors,
// pivots and INFO are those of the reference's column-by-column PDGETF2 in
// exact arithmetic.
#include <climits>
#include <cuda_runtime.h>
#include <stdint.h>
#include "common.cuh"
#include "sl_internal.h"

namespace sl {

constexpr int PW = 32;       // sub-panel width held in shared memory
constexpr int PMAXG = 1024;  // max CTAs of the panel kernel
constexpr int PT = 256;      // threads per panel CTA
constexpr int PLD = PW + 1;  // shared row stride (doubles): conflict-free row/column walks

size_t panel_cand_doubles() { return (size_t)2 * PMAXG * (PW + 2) + 2 * PW; }
static_assert(kPanelCandDoubles == (size_t)2 * PMAXG * (PW + 2) + 2 * PW, "slot layout");

// Rows per CTA are capped by 200 KB of shared memory (rpc * 33 doubles),
// rounded down to a multiple of 8: 768 rows; one CTA per SM.
int panel_max_rows() { return num_sms() * 768; }

// Factor rows [r0, m) x columns [c0, c0+w) (w <= 32) of A in place.
// Writes ipiv[c0+k] = 0-based pivot row for k < min(w, m-r0); records the first
// exactly-zero pivot column in *info_col. Row interchanges are applied to the
// w sub-panel columns only.
__global__ void __launch_bounds__(PT)
panel_f64_kernel(double* A, long long lda, int m, int r0, int c0, int w, int rpc, int* ipiv,
                 int* info_col, double* cand, int* bar, int* status) {
  extern __shared__ double tile[];  // [rpc][PLD]
  __shared__ double s_U[PW], s_D[PW];
  __shared__ double s_wk[PT / 32];
  __shared__ int s_wr[PT / 32];
  __shared__ int s_row;
  __shared__ int s_piv;
  __shared__ double s_gmax;

  const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const int R = m - r0;
  const int kw = min(w, R);
  const int lo = b * rpc;                       // first local row (relative to r0)
  const int nr = max(0, min(rpc, R - lo));      // rows owned
  double* diag = cand + (size_t)2 * PMAXG * (PW + 2);

  for (int c = 0; c < w; ++c)
    for (int r = tid; r < nr; r += PT)
      tile[r * PLD + c] = A[(long long)(r0 + lo + r) + (long long)(c0 + c) * lda];
  __syncthreads();

  for (int k = 0; k < kw; ++k) {
    const int d = k;  // diagonal row relative to r0
    const int par = k & 1;
    // --- local IDAMAX over owned rows >= d ---
    double key = -2.0;
    int row = INT_MAX;
    for (int r = tid; r < nr; r += PT) {
      int gr = lo + r;
      if (gr >= d) amax_combine(key, row, amax_key(tile[r * PLD + k]), gr);
    }
    warp_amax(key, row);
    if (lane == 0) { s_wk[warp] = key; s_wr[warp] = row; }
    __syncthreads();
    if (warp == 0) {
      key = lane < PT / 32 ? s_wk[lane] : -2.0;
      row = lane < PT / 32 ? s_wr[lane] : INT_MAX;
      warp_amax(key, row);
      if (lane == 0) {
        s_row = row;
        double* slot = cand + ((size_t)par * PMAXG + b) * (PW + 2);
        slot[0] = key;
        slot[1] = (double)row;
      }
    }
    __syncthreads();
    {
      double* slot = cand + ((size_t)par * PMAXG + b) * (PW + 2);
      int lr = s_row;
      if (tid < w && lr != INT_MAX) slot[2 + tid] = tile[(lr - lo) * PLD + tid];
      if (d >= lo && d < lo + nr && tid < w) diag[par * PW + tid] = tile[(d - lo) * PLD + tid];
    }
    __threadfence();
    if (!grid_barrier(bar, G, status)) return;

    // --- global winner (largest |x|, lowest row on ties) ---
    key = -2.0;
    row = INT_MAX;
    for (int q = tid; q < G; q += PT) {
      const double* slot = cand + ((size_t)par * PMAXG + q) * (PW + 2);
      double k2 = __ldcg(slot);
      double r2 = __ldcg(slot + 1);
      int ri = (r2 >= (double)INT_MAX) ? INT_MAX : (int)r2;
      amax_combine(key, row, k2, ri);
    }
    warp_amax(key, row);
    if (lane == 0) { s_wk[warp] = key; s_wr[warp] = row; }
    __syncthreads();
    if (warp == 0) {
      key = lane < PT / 32 ? s_wk[lane] : -2.0;
      row = lane < PT / 32 ? s_wr[lane] : INT_MAX;
      warp_amax(key, row);
      if (lane == 0) { s_row = row; s_wk[0] = key; }
    }
    __syncthreads();
    const int grow = s_row;
    const double gkey = s_wk[0];
    if (tid < w) s_D[tid] = __ldcg(diag + par * PW + tid);
    __syncthreads();
    if (tid == 0) {
      // IDAMAX keeps the first element when it is NaN; AMAX == 0 selects the
      // diagonal row (PBLAS/SRC/pdamax_.c:486).
      int piv = grow;
      double dv = s_D[k];
      if (dv != dv || gkey == 0.0) piv = d;
      s_piv = piv;
    }
    __syncthreads();
    const int piv = s_piv;
    if (tid < w) {
      if (piv == d) s_U[tid] = s_D[tid];
      else {
        int wb = piv / rpc;
        s_U[tid] = __ldcg(cand + ((size_t)par * PMAXG + wb) * (PW + 2) + 2 + tid);
      }
    }
    __syncthreads();
    if (tid == 0) s_gmax = s_U[k];
    // --- row interchange inside the sub-panel (PDSWAP, pdgetf2.f:218) ---
    if (piv != d && tid < w) {
      if (d >= lo && d < lo + nr) tile[(d - lo) * PLD + tid] = s_U[tid];
      if (piv >= lo && piv < lo + nr) tile[(piv - lo) * PLD + tid] = s_D[tid];
    }
    __syncthreads();
    const double gmax = s_gmax;
    if (b == 0 && tid == 0) {
      ipiv[c0 + k] = r0 + piv;
      if (gmax == 0.0) atomicMin(info_col, c0 + k);
    }
    // --- scale by ONE/GMAX (PDSCAL, pdgetf2.f:224) and rank-1 update (PDGER) ---
    const bool scale = (gmax != 0.0);
    const double rinv = scale ? 1.0 / gmax : 0.0;
    for (int r = warp; r < nr; r += PT / 32) {
      int gr = lo + r;
      if (gr <= d) continue;
      double l = tile[r * PLD + k];
      if (scale) l *= rinv;
      __syncwarp();
      if (lane == k) tile[r * PLD + k] = l;
      else if (lane > k && lane < w) tile[r * PLD + lane] = fma(-l, s_U[lane], tile[r * PLD + lane]);
    }
    __syncthreads();
  }

  for (int c = 0; c < w; ++c)
    for (int r = tid; r < nr; r += PT)
      A[(long long)(r0 + lo + r) + (long long)(c0 + c) * lda] = tile[r * PLD + c];
}

// Sequential row interchanges k1..k2-1 (rows i <-> ipiv[i]) on the columns
// [cb1,ce1) and [cb2,ce2); one thread per column (PDLASWP 'Forward','Rows').
__global__ void __launch_bounds__(256)
laswp_kernel(double* A, long long lda, int k1, int k2, const int* __restrict__ ipiv, int cb1,
             int ce1, int cb2, int ce2) {
  __shared__ int s_piv[1024];
  const int npiv = k2 - k1;
  for (int i = threadIdx.x; i < npiv && i < 1024; i += blockDim.x) s_piv[i] = ipiv[k1 + i];
  __syncthreads();
  const long long n1 = ce1 - cb1, n2 = ce2 - cb2;
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n1 + n2) return;
  long long col = idx < n1 ? cb1 + idx : cb2 + (idx - n1);
  double* a = A + col * lda;
  for (int i = 0; i < npiv; ++i) {
    int p = i < 1024 ? s_piv[i] : ipiv[k1 + i];
    int r = k1 + i;
    if (p != r) {
      double t = a[r];
      a[r] = a[p];
      a[p] = t;
    }
  }
}

// op(T) X = B for a w x w triangle T (w <= 256) and a strip of NC columns of B
// per CTA, in shared memory. FORWARD solves top-down (lower, or upper^T),
// otherwise bottom-up. Non-unit diagonals divide (reference DTRSM semantics).
template <bool UPPER, bool TRANS, bool UNIT, int NC>
__global__ void __launch_bounds__(256)
trsm_strip_kernel(int w, int ncols, const double* __restrict__ T, long long ldt, double* B,
                  long long ldb) {
  constexpr bool FORWARD = (UPPER == TRANS);
  constexpr int RG = 256 / NC;  // row groups
  extern __shared__ double Bs[];  // [w][NC+1]
  const int LD = NC + 1;
  const int tid = threadIdx.x;
  const int c = tid % NC, rg = tid / NC;
  const long long col0 = (long long)blockIdx.x * NC;
  const int nc = (int)min((long long)NC, ncols - col0);
  for (int i = tid; i < w * NC; i += 256) {
    int r = i % w, cc = i / w;
    Bs[r * LD + cc] = cc < nc ? B[r + (col0 + cc) * ldb] : 0.0;
  }
  __syncthreads();
  auto E = [&](int i, int j) -> double {
    return TRANS ? T[j + (long long)i * ldt] : T[i + (long long)j * ldt];
  };
  for (int s = 0; s < w; ++s) {
    const int i = FORWARD ? s : w - 1 - s;
    if (!UNIT) {
      if (tid < NC) Bs[i * LD + tid] = Bs[i * LD + tid] / E(i, i);
      __syncthreads();
    }
    const double xi = Bs[i * LD + c];
    if (FORWARD) {
      for (int r = i + 1 + rg; r < w; r += RG) Bs[r * LD + c] = fma(-E(r, i), xi, Bs[r * LD + c]);
    } else {
      for (int r = rg; r < i; r += RG) Bs[r * LD + c] = fma(-E(r, i), xi, Bs[r * LD + c]);
    }
    __syncthreads();
  }
  for (int i = tid; i < w * NC; i += 256) {
    int r = i % w, cc = i / w;
    if (cc < nc) B[r + (col0 + cc) * ldb] = Bs[r * LD + cc];
  }
}

template <bool UPPER, bool TRANS, bool UNIT>
static cudaError_t trsm_strip(int w, int ncols, const double* T, long long ldt, double* B,
                              long long ldb, cudaStream_t s) {
  if (w <= 0 || ncols <= 0) return cudaSuccess;
  constexpr int NC = 8;
  size_t smem = sizeof(double) * (size_t)w * (NC + 1);
  auto kern = trsm_strip_kernel<UPPER, TRANS, UNIT, NC>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
  }
  dim3 grid((ncols + NC - 1) / NC);
  kern<<<grid, 256, smem, s>>>(w, ncols, T, ldt, B, ldb);
  count_launches(1);
  return cudaGetLastError();
}

// Composed row permutation of the n sequential interchanges i <-> ipiv[i]:
// perm[i] = original row that ends in row i. One CTA, the walk in shared
// memory (n <= smem_cap) or in global memory otherwise.
__global__ void perm_compose_kernel(const int* __restrict__ ipiv, int n, int* perm, int use_smem) {
  extern __shared__ int sp[];
  int* p = use_smem ? sp : perm;
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = i;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) {
      int q = ipiv[i];
      if (q != i) {
        int t = p[i];
        p[i] = p[q];
        p[q] = t;
      }
    }
  }
  __syncthreads();
  if (use_smem)
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = sp[i];
}

// dst(i, c) = src(perm[i], c) (forward) or dst(perm[i], c) = src(i, c) (inverse).
__global__ void permute_rows_kernel(const double* __restrict__ src, long long lds, double* dst,
                                    long long ldd, const int* __restrict__ perm, int n, int nrhs,
                                    int inverse) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * nrhs) return;
  int i = (int)(idx % n), c = (int)(idx / n);
  int p = perm[i];
  if (!inverse) dst[i + c * ldd] = src[p + c * lds];
  else dst[p + c * ldd] = src[i + c * lds];
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

static cudaError_t launch_panel(double* A, long long lda, int m, int r0, int c0, int w, int* ipiv,
                                const LuWork& ws, cudaStream_t s) {
  const int R = m - r0;
  const int nsm = num_sms();
  int rpc = (R + nsm - 1) / nsm;
  if (rpc < 64) rpc = 64;
  rpc = (rpc + 7) & ~7;
  int G = (R + rpc - 1) / rpc;
  size_t smem = sizeof(double) * (size_t)rpc * PLD;
  if (smem > 200 * 1024 || G > PMAXG) return cudaErrorInvalidValue;  // M beyond the panel limit
  static size_t smem_set = 0;
  if (smem > 48 * 1024 && smem > smem_set) {
    cudaError_t e = cudaFuncSetAttribute(panel_f64_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    smem_set = 200 * 1024;
  }
  cudaError_t e = cudaMemsetAsync(ws.bar, 0, 2 * sizeof(int), s);
  if (e != cudaSuccess) return e;
  void* args[] = {&A, &lda, &m, &r0, &c0, &w, &rpc, &ipiv, (void*)&ws.info_col, (void*)&ws.cand,
                  (void*)&ws.bar, (void*)&ws.status};
  count_launches(1);
  return cudaLaunchCooperativeKernel((void*)panel_f64_kernel, dim3(G), dim3(PT), args, smem, s);
}

static cudaError_t laswp(double* A, long long lda, int k1, int k2, const int* ipiv, int cb1,
                         int ce1, int cb2, int ce2, cudaStream_t s) {
  long long ncols = (long long)(ce1 - cb1) + (ce2 - cb2);
  if (ncols <= 0 || k2 <= k1) return cudaSuccess;
  dim3 grid((unsigned)((ncols + 255) / 256));
  laswp_kernel<<<grid, 256, 0, s>>>(A, lda, k1, k2, ipiv, cb1, ce1, cb2, ce2);
  count_launches(1);
  return cudaGetLastError();
}

#define SL_TRY(x)                        \
  do {                                   \
    cudaError_t _e = (x);                \
    if (_e != cudaSuccess) return _e;    \
  } while (0)

cudaError_t dgetrf_device(int m, int n, double* dA, long long ldda, int* dipiv, int nb,
                          const LuWork& ws, cudaStream_t s) {
  SL_TRY(cudaMemsetAsync(ws.status, 0, sizeof(int), s));
  SL_TRY(cudaMemsetAsync(ws.info_col, 0x7f, sizeof(int), s));
  const int mn = m < n ? m : n;
  if (nb > 1024) nb = 1024;
  auto Ap = [&](long long i, long long j) { return dA + i + j * ldda; };
  for (int j = 0; j < mn; j += nb) {
    const int jb = (mn - j) < nb ? (mn - j) : nb;
    // ---- panel (PDGETF2) as 32-wide sub-panels ----
    phase_begin(kPhPanel, s);
    double pflops = 0.0;
    for (int c = 0; c < jb; c += PW) {
      const int w = (jb - c) < PW ? (jb - c) : PW;
      const int r0 = j + c;
      SL_TRY(launch_panel(dA, ldda, m, r0, r0, w, dipiv, ws, s));
      const int kw = (m - r0) < w ? (m - r0) : w;
      for (int k = 0; k < kw; ++k) pflops += 2.0 * (double)(m - r0 - k - 1) * (w - k - 1) + (m - r0 - k - 1);
      SL_TRY(laswp(dA, ldda, r0, r0 + kw, dipiv, j, r0, r0 + w, j + jb, s));
      if (c + w < jb) {
        SL_TRY((trsm_strip<false, false, true>(kw, jb - c - w, Ap(r0, r0), ldda, Ap(r0, r0 + w),
                                               ldda, s)));
        pflops += (double)kw * kw * (jb - c - w);
        if (r0 + kw < m) {
          SL_TRY(dgemm(false, m - r0 - kw, jb - c - w, kw, -1.0, Ap(r0 + kw, r0), ldda,
                       Ap(r0, r0 + w), ldda, 1.0, Ap(r0 + kw, r0 + w), ldda, s));
          pflops += 2.0 * (double)(m - r0 - kw) * (jb - c - w) * kw;
        }
      }
    }
    phase_end(kPhPanel, s, pflops, 16.0 * (double)(m - j) * jb);
    // ---- PDLASWP on the left and right column blocks ----
    phase_begin(kPhLaswp, s);
    SL_TRY(laswp(dA, ldda, j, j + jb, dipiv, 0, j, j + jb, n, s));
    phase_end(kPhLaswp, s, 0.0, 32.0 * jb * (double)(n - jb));
    if (j + jb < n) {
      // ---- PDTRSM: U12 = L11^{-1} A12 ----
      const double nr = (double)(n - j - jb);
      phase_begin(kPhTrsm, s);
      SL_TRY((trsm_strip<false, false, true>(jb, n - j - jb, Ap(j, j), ldda, Ap(j, j + jb), ldda,
                                             s)));
      phase_end(kPhTrsm, s, (double)jb * jb * nr, 8.0 * (0.5 * jb * jb + 2.0 * jb * nr));
      // ---- PDGEMM: A22 -= L21 * U12 ----
      if (j + jb < m) {
        const double mr = (double)(m - j - jb);
        phase_begin(kPhGemm, s);
        SL_TRY(dgemm(false, m - j - jb, n - j - jb, jb, -1.0, Ap(j + jb, j), ldda, Ap(j, j + jb),
                     ldda, 1.0, Ap(j + jb, j + jb), ldda, s));
        phase_end(kPhGemm, s, 2.0 * mr * nr * jb, 8.0 * (mr * jb + jb * nr + 2.0 * mr * nr));
      }
    }
  }
  return cudaGetLastError();
}

// Blocked triangular solve with the n x n factors for nrhs columns of X:
// diagonal 64-blocks with the strip kernel, off-diagonal updates with dgemm.
static cudaError_t tri_solve(bool lower, bool trans, bool unit, int n, int nrhs, const double* A,
                             long long lda, double* X, long long ldx, cudaStream_t s) {
  const int KB = 64;
  // effective lower (forward) when lower&&!trans or upper&&trans
  const bool forward = (lower != trans);
  const int nblk = (n + KB - 1) / KB;
  for (int bi = 0; bi < nblk; ++bi) {
    const int b = forward ? bi : nblk - 1 - bi;
    const int k0 = b * KB;
    const int kb = (n - k0) < KB ? (n - k0) : KB;
    const double* Td = A + k0 + (long long)k0 * lda;
    if (lower && !trans) SL_TRY((trsm_strip<false, false, true>(kb, nrhs, Td, lda, X + k0, ldx, s)));
    else if (!lower && !trans) {
      if (unit) SL_TRY((trsm_strip<true, false, true>(kb, nrhs, Td, lda, X + k0, ldx, s)));
      else SL_TRY((trsm_strip<true, false, false>(kb, nrhs, Td, lda, X + k0, ldx, s)));
    } else if (!lower && trans) SL_TRY((trsm_strip<true, true, false>(kb, nrhs, Td, lda, X + k0, ldx, s)));
    else SL_TRY((trsm_strip<false, true, true>(kb, nrhs, Td, lda, X + k0, ldx, s)));
    (void)unit;
    if (forward) {
      const int rest = n - k0 - kb;
      if (rest > 0) {
        // X[k0+kb:] -= op(T)[k0+kb:, k0:k0+kb] * X[k0:k0+kb]
        const double* Aoff = trans ? A + k0 + (long long)(k0 + kb) * lda   // (T^T) block = T[k0.., k0+kb..]^T
                                   : A + (k0 + kb) + (long long)k0 * lda;
        SL_TRY(dgemm(trans, rest, nrhs, kb, -1.0, Aoff, lda, X + k0, ldx, 1.0, X + k0 + kb, ldx, s));
      }
    } else {
      if (k0 > 0) {
        // X[0:k0] -= op(T)[0:k0, k0:k0+kb] * X[k0:k0+kb]
        const double* Aoff = trans ? A + k0 : A + (long long)k0 * lda;
        SL_TRY(dgemm(trans, k0, nrhs, kb, -1.0, Aoff, lda, X + k0, ldx, 1.0, X, ldx, s));
      }
    }
  }
  return cudaSuccess;
}

cudaError_t dgetrs_device(char trans, int n, int nrhs, const double* dA, long long ldda,
                          const int* dipiv, double* dB, long long lddb, const LuWork& ws,
                          cudaStream_t s) {
  if (n <= 0 || nrhs <= 0) return cudaSuccess;
  const bool notran = (trans == 'N' || trans == 'n');
  phase_begin(kPhSolve, s);
  // composed permutation of the n interchanges (PDLAPIV)
  const size_t smem = sizeof(int) * (size_t)n;
  const int use_smem = smem <= 200 * 1024 ? 1 : 0;
  if (use_smem && smem > 48 * 1024)
    SL_TRY(cudaFuncSetAttribute(perm_compose_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                200 * 1024));
  perm_compose_kernel<<<1, 1024, use_smem ? smem : 0, s>>>(dipiv, n, ws.perm, use_smem);
  count_launches(1);
  SL_TRY(cudaGetLastError());
  double* X = ws.bswap;  // n x nrhs, ld = n
  const long long total = (long long)n * nrhs;
  const unsigned pg = (unsigned)((total + 255) / 256);
  if (notran) {
    permute_rows_kernel<<<pg, 256, 0, s>>>(dB, lddb, X, n, ws.perm, n, nrhs, 0);
    count_launches(1);
    SL_TRY(cudaGetLastError());
    SL_TRY(tri_solve(true, false, true, n, nrhs, dA, ldda, X, n, s));
    SL_TRY(tri_solve(false, false, false, n, nrhs, dA, ldda, X, n, s));
    SL_TRY(cudaMemcpy2DAsync(dB, lddb * sizeof(double), X, n * sizeof(double),
                             n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s));
  } else {
    SL_TRY(cudaMemcpy2DAsync(X, n * sizeof(double), dB, lddb * sizeof(double),
                             n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s));
    SL_TRY(tri_solve(false, true, false, n, nrhs, dA, ldda, X, n, s));
    SL_TRY(tri_solve(true, true, true, n, nrhs, dA, ldda, X, n, s));
    permute_rows_kernel<<<pg, 256, 0, s>>>(X, n, dB, lddb, ws.perm, n, nrhs, 1);
    count_launches(1);
    SL_TRY(cudaGetLastError());
  }
  phase_end(kPhSolve, s, 2.0 * (double)n * n * nrhs, 8.0 * ((double)n * n + 4.0 * (double)n * nrhs));
  return cudaSuccess;
}

}  // namespace sl
