// Mixed-precision LU with iterative refinement (LU-IR) on one GB300.
//
// Factorization (the PDGETRF loop of SRC/pdgetrf.f:254-295 in low precision):
// the FP64 matrix is copied to an FP32 working matrix; the panel (PDGETF2),
// row interchanges (PDLASWP) and U12 solve (PDTRSM) run in FP32 with the same
// kernels as the FP64 path, and the trailing update (PDGEMM) rounds L21 and
// U12 to BF16 or FP16 -- U12 scaled per column by a power of two -- and
// multiplies them on tcgen05 tensor cores with FP32 accumulation
// (mixed_gemm.cu).
//
// Refinement: FP64 is kept only for the residual b - A x (the original FP64
// matrix stays untouched in HBM), the solution update and the GMRES
// orthogonalization. Corrections are solved with the FP32 factors (right-hand
// side scaled by a power of two into FP32 range). Classical refinement runs up
// to `max_ir` steps and stops when the tester's scaled residual
// ||b - A x||_inf / (||A||_inf ||x||_inf N eps) (TESTING/traditional/LIN/
// pdlaschk.f:185-187) is at or below `tol`; when a step fails to halve it,
// GMRES-IR takes over (GMRES on the left-preconditioned system (LU)^-1 A d =
// (LU)^-1 r, classical Gram-Schmidt applied twice, Givens rotations). When
// GMRES-IR also stalls, the plain FP64 factorization (dgetrf_device) is run and the
// system is solved in plain FP64 (the reference's PDGERFS stall rule,
// SRC/pdgerfs.f:552, motivates the halving test).
#include <cuda_runtime.h>

#include <chrono>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "lu_kernels.cuh"
#include "sl_internal.h"

namespace sl {

// ------------------------------------------------------------ FP32 SIMT GEMM
// C (m x n) += alpha op(A) (m x k) B (k x n), FP32, column-major. 64x64 tiles,
// K-step 16, 256 threads each computing 4x4. Used for the in-panel updates of
// the FP32 factorization (k = 32) and for wide right-hand sides in the solves.
template <bool TRANSA>
__global__ void __launch_bounds__(256)
sgemm_simt_kernel(int m, int n, int k, float alpha, const float* __restrict__ A, long long lda,
                  const float* __restrict__ B, long long ldb, float* C, long long ldc) {
  __shared__ float As[16][64 + 4];
  __shared__ float Bs[16][64 + 4];
  const int tid = threadIdx.x;
  const int tx = tid % 16, ty = tid / 16;
  const long long m0 = (long long)blockIdx.x * 64, n0 = (long long)blockIdx.y * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < k; k0 += 16) {
    for (int c = tid; c < 64 * 16; c += 256) {
      int mm, kk;
      if (!TRANSA) { kk = c / 64; mm = c % 64; } else { mm = c / 16; kk = c % 16; }
      long long gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < m && gk < k) ? (TRANSA ? A[gk + gm * lda] : A[gm + gk * lda]) : 0.f;
      int nn = c / 16, kb = c % 16;
      long long gn = n0 + nn, gkb = k0 + kb;
      Bs[kb][nn] = (gn < n && gkb < k) ? B[gkb + gn * ldb] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      long long r = m0 + ty * 4 + i, c = n0 + tx * 4 + j;
      if (r < m && c < n) C[r + c * ldc] += alpha * acc[i][j];
    }
}

static cudaError_t sgemm_simt(bool transa, int m, int n, int k, float alpha, const float* A,
                              long long lda, const float* B, long long ldb, float* C,
                              long long ldc, cudaStream_t s) {
  if (m <= 0 || n <= 0 || k <= 0) return cudaSuccess;
  dim3 grid((m + 63) / 64, (n + 63) / 64);
  if (transa) sgemm_simt_kernel<true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, C, ldc);
  else sgemm_simt_kernel<false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, C, ldc);
  count_launches(1);
  return cudaGetLastError();
}

template <>
cudaError_t gemm_update<float>(bool transa, int m, int n, int k, float alpha, const float* A,
                               long long lda, const float* B, long long ldb, float* C,
                               long long ldc, cudaStream_t s) {
  if (n <= 16) return gemm_skinny<float>(transa, m, n, k, alpha, A, lda, B, ldb, C, ldc, s);
  return sgemm_simt(transa, m, n, k, alpha, A, lda, B, ldb, C, ldc, s);
}

// ------------------------------------------------------------ small kernels
__global__ void d2s_kernel(const double* __restrict__ A, long long lda, int m, int n, float* F,
                           long long ldf) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long total = (long long)m * n;
  for (; idx < total; idx += (long long)gridDim.x * blockDim.x) {
    int i = (int)(idx % m);
    long long j = idx / m;
    F[i + j * ldf] = (float)A[i + j * lda];
  }
}

// out[c] = max_i |X(i,c)| (NaN propagates), one CTA per column.
__global__ void colmax_abs_kernel(const double* __restrict__ X, long long ldx, int n, double* out) {
  __shared__ double sm[32];
  const int c = blockIdx.x;
  double mx = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double v = fabs(X[i + (long long)c * ldx]);
    mx = (v > mx || v != v) ? v : mx;
  }
  for (int off = 16; off > 0; off >>= 1) {
    double o = __shfl_xor_sync(0xffffffffu, mx, off);
    mx = (o > mx || o != o) ? o : mx;
  }
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    mx = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) {
      double o = __shfl_xor_sync(0xffffffffu, mx, off);
      mx = (o > mx || o != o) ? o : mx;
    }
    if (threadIdx.x == 0) out[c] = mx;
  }
}

// ||A||_inf = max_i sum_j |A(i,j)|: row sums by threads over rows.
__global__ void rowsum_abs_kernel(const double* __restrict__ A, long long lda, int n,
                                  double* rows) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int j = 0; j < n; ++j) s += fabs(A[i + (long long)j * lda]);
  rows[i] = s;
}

// Fx(:,c) = float(R(:,c) * 2^-e_c) with e_c the exponent of colmax[c].
__global__ void scale_to_float_kernel(const double* __restrict__ R, long long ldr, int n, int ncols,
                                      const double* __restrict__ colmax, float* Fx,
                                      long long ldf) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * ncols) return;
  int i = (int)(idx % n), c = (int)(idx / n);
  int e = 0;
  double mx = colmax[c];
  if (mx > 0.0 && isfinite(mx)) frexp(mx, &e);
  Fx[i + (long long)c * ldf] = (float)ldexp(R[i + (long long)c * ldr], -e);
}

// X(:,c) = beta * X(:,c) + double(Fx(:,c)) * 2^e_c.
__global__ void float_scaled_add_kernel(const float* __restrict__ Fx, long long ldf, int n,
                                        int ncols, const double* __restrict__ colmax, double beta,
                                        double* X, long long ldx) {
  long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * ncols) return;
  int i = (int)(idx % n), c = (int)(idx / n);
  int e = 0;
  double mx = colmax[c];
  if (mx > 0.0 && isfinite(mx)) frexp(mx, &e);
  double v = ldexp((double)Fx[i + (long long)c * ldf], e);
  double* xp = X + i + (long long)c * ldx;
  *xp = (beta == 0.0) ? v : beta * *xp + v;
}

// h[i] = V(:,i) . w for i < ncols (one CTA per column, fixed reduction order).
__global__ void dots_kernel(const double* __restrict__ V, long long ldv, int n, int ncols,
                            const double* __restrict__ w, double* h) {
  __shared__ double sm[32];
  const int c = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(V[i + (long long)c * ldv], w[i], s);
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (threadIdx.x == 0) h[c] = s;
  }
}

// w -= V(:, 0:ncols) h
__global__ void sub_vh_kernel(const double* __restrict__ V, long long ldv, int n, int ncols,
                              const double* __restrict__ h, double* w) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = w[i];
  for (int c = 0; c < ncols; ++c) s = fma(-V[i + (long long)c * ldv], h[c], s);
  w[i] = s;
}

// y = alpha * x (n entries), alpha read from device memory as 1/alpha_inv.
__global__ void scale_vec_kernel(const double* __restrict__ x, int n, const double* alpha_inv,
                                 double* y) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] / alpha_inv[0];
}

// x += V(:,0:k) y (host-supplied coefficients in device memory).
__global__ void add_vy_kernel(const double* __restrict__ V, long long ldv, int n, int k,
                              const double* __restrict__ y, double* x) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = x[i];
  for (int c = 0; c < k; ++c) s = fma(V[i + (long long)c * ldv], y[c], s);
  x[i] = s;
}

// y += x
__global__ void axpy1_kernel(int n, const double* __restrict__ x, double* y) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += x[i];
}

static unsigned blocks_for(long long n, int t = 256) {
  long long b = (n + t - 1) / t;
  return (unsigned)(b < 1 ? 1 : b);
}

// ---------------------------------------------------- FP32 factorization
// PDGETF2 in FP32 on columns [j, j+jb), rows [j, n).
static cudaError_t factor_panel_f32(int n, float* F, long long ldf, int* dipiv, int j, int jb,
                                    const LuWork& ws, cudaStream_t s) {
  auto Fp = [&](long long i, long long c) { return F + i + c * ldf; };
  const int m = n;
  phase_begin(kPhMixedPanel, s);
  for (int c = 0; c < jb; c += PW) {
    const int w = (jb - c) < PW ? (jb - c) : PW;
    const int r0 = j + c;
    SL_TRY(launch_panel<float>(F, ldf, m, r0, r0, w, dipiv, ws, s));
    const int kw = (m - r0) < w ? (m - r0) : w;
    SL_TRY(laswp<float>(F, ldf, r0, r0 + kw, dipiv, j, r0, r0 + w, j + jb, s));
    if (c + w < jb) {
      SL_TRY((trsm_strip<float, false, false, true>(kw, jb - c - w, Fp(r0, r0), ldf,
                                                     Fp(r0, r0 + w), ldf, s)));
      if (r0 + kw < m)
        SL_TRY(sgemm_simt(false, m - r0 - kw, jb - c - w, kw, -1.f, Fp(r0 + kw, r0), ldf,
                          Fp(r0, r0 + w), ldf, Fp(r0 + kw, r0 + w), ldf, s));
    }
  }
  const int npiv = (m - j) < jb ? (m - j) : jb;
  if (ws.swap_plan && npiv <= LSW_MAXP) SL_TRY(laswp_plan(j, j + npiv, dipiv, ws.swap_plan, s));
  phase_end(kPhMixedPanel, s, 0.0, 0.0);
  return cudaSuccess;
}

// Low-precision right-looking LU of the FP32 working matrix, with the same
// look-ahead as the FP64 path (next panel on ws.aux while the tcgen05 update
// of the remaining columns runs).
cudaError_t sgetrf_mixed_device(int n, float* F, long long ldf, int* dipiv, int nb, int fmt,
                                const LuWork& ws, const MixedWork& mw, cudaStream_t s) {
  SL_TRY(cudaMemsetAsync(ws.status, 0, sizeof(int), s));
  SL_TRY(cudaMemsetAsync(ws.info_col, 0x7f, sizeof(int), s));
  const int m = n, mn = n;
  if (nb > 1024) nb = 1024;
  auto Fp = [&](long long i, long long j) { return F + i + j * ldf; };
  const bool lookahead = ws.aux && ws.ev_next && ws.ev_panel && mn > 2 * nb;
  if (mn > 0) SL_TRY(factor_panel_f32(n, F, ldf, dipiv, 0, (mn < nb ? mn : nb), ws, s));
  bool panel_on_aux = false;
  for (int j = 0; j < mn; j += nb) {
    const int jb = (mn - j) < nb ? (mn - j) : nb;
    if (panel_on_aux) SL_TRY(cudaStreamWaitEvent(s, ws.ev_panel, 0));
    panel_on_aux = false;
    const int jn = j + jb;
    const int jb2 = jn < mn ? ((mn - jn) < nb ? (mn - jn) : nb) : 0;
    phase_begin(kPhMixedPanel, s);
    SL_TRY(laswp_planned<float>(F, ldf, j, j + jb, dipiv, ws.swap_plan, 0, j, j + jb, n, s));
    if (jn < n)
      SL_TRY((trsm_strip<float, false, false, true>(jb, n - jn, Fp(j, j), ldf, Fp(j, jn), ldf, s)));
    phase_end(kPhMixedPanel, s, 0.0, 0.0);
    if (jn < n && jn < m) {
      const int mr = m - jn, nr = n - jn;
      const int kp = lowp_kpad(jb) * lowp_kmult(fmt);
      phase_begin(kPhMixedGemm, s);
      SL_TRY(lowp_pack(fmt, Fp(jn, j), ldf, mr, Fp(j, jn), ldf, nr, jb, mw.A16, mw.B16, mw.col_exp, s));
      if (lookahead && jb2 > 0) {
        SL_TRY(lowp_gemm(fmt, mr, jb2, jb, mw.A16, mw.B16, mw.col_exp, Fp(jn, jn), ldf, ws.status, s));
        phase_end(kPhMixedGemm, s, 2.0 * mr * (double)jb2 * jb, 8.0 * (double)mr * jb2);
        SL_TRY(cudaEventRecord(ws.ev_next, s));
        SL_TRY(cudaStreamWaitEvent(ws.aux, ws.ev_next, 0));
        SL_TRY(factor_panel_f32(n, F, ldf, dipiv, jn, jb2, ws, ws.aux));
        SL_TRY(cudaEventRecord(ws.ev_panel, ws.aux));
        panel_on_aux = true;
        const int rest = nr - jb2;
        if (rest > 0) {
          phase_begin(kPhMixedGemm, s);
          SL_TRY(lowp_gemm(fmt, mr, rest, jb, mw.A16, mw.B16 + (long long)jb2 * kp, mw.col_exp + jb2,
                           Fp(jn, jn + jb2), ldf, ws.status, s));
          phase_end(kPhMixedGemm, s, 2.0 * mr * (double)rest * jb,
                    8.0 * (double)mr * rest + 2.0 * ((double)mr + rest) * kp);
        }
      } else {
        SL_TRY(lowp_gemm(fmt, mr, nr, jb, mw.A16, mw.B16, mw.col_exp, Fp(jn, jn), ldf, ws.status, s));
        phase_end(kPhMixedGemm, s, 2.0 * mr * (double)nr * jb,
                  8.0 * (double)mr * nr + 2.0 * ((double)mr + nr) * kp);
      }
    }
    if (jb2 > 0 && !panel_on_aux) SL_TRY(factor_panel_f32(n, F, ldf, dipiv, jn, jb2, ws, s));
  }
  if (panel_on_aux) SL_TRY(cudaStreamWaitEvent(s, ws.ev_panel, 0));
  return cudaGetLastError();
}

// Inverses of the 64x64 diagonal blocks of the FP32 factors for the chained
// solves: block b of L (unit lower, LOWER) or U (non-unit upper) is inverted
// column by column (thread t solves T x = e_t by substitution, accumulating in
// FP64) and stored row-major at Dinv[b*64*64 + r*64 + i]; a partial last block
// is padded with the identity. Also M_b = inv(T_bb) T_bp, with p the block
// solved just before b (b-1 for L, b+1 for U; zero for the first one), stored
// the same way at Mp: the chained solve then finishes block b with one 64x64
// product once x_p arrives, x_b = inv(T_bb) v_b - M_b x_p.
template <bool LOWER>
__global__ void __launch_bounds__(64)
diag_inv_kernel(int n, const float* __restrict__ F, long long ldf, float* Dinv, float* Mp) {
  constexpr int KB = 64;
  __shared__ float T[KB][KB];   // read as broadcasts: no padding needed
  __shared__ double X[KB][KB];  // X[i][t]: column t of the inverse (thread t's own column)
  const int b = blockIdx.x, t = threadIdx.x;
  const int r0 = b * KB, rb = min(KB, n - r0);
  for (int r = 0; r < KB; ++r) {
    const int i = t;
    const bool in = r < rb && i < rb && (LOWER ? i < r : i >= r);
    T[r][i] = in ? F[(r0 + r) + (long long)(r0 + i) * ldf] : (r == i ? 1.0f : 0.0f);
  }
  __syncthreads();
  if (LOWER) {
    for (int i = 0; i < KB; ++i) {
      double acc = (i == t) ? 1.0 : 0.0;
      for (int j = t; j < i; ++j) acc -= (double)T[i][j] * X[j][t];
      X[i][t] = (i < t) ? 0.0 : acc;
    }
  } else {
    for (int i = KB - 1; i >= 0; --i) {
      double acc = (i == t) ? 1.0 : 0.0;
      for (int j = i + 1; j <= t; ++j) acc -= (double)T[i][j] * X[j][t];
      X[i][t] = (i > t) ? 0.0 : acc / (double)T[i][i];
    }
  }
  __syncthreads();
  float* D = Dinv + (size_t)b * KB * KB;
  for (int r = 0; r < KB; ++r) D[r * KB + t] = (float)X[r][t];
  // the predecessor block into T (its triangle is no longer needed)
  const int nblk = (n + KB - 1) / KB;
  const int p = LOWER ? b - 1 : b + 1;
  const bool has_p = p >= 0 && p < nblk;
  const int wp = has_p ? min(KB, n - p * KB) : 0;
  for (int r = 0; r < KB; ++r)
    T[r][t] = (r < rb && t < wp) ? F[(r0 + r) + (long long)(p * KB + t) * ldf] : 0.0f;
  __syncthreads();
  float* M = Mp + (size_t)b * KB * KB;
  for (int r = 0; r < KB; ++r) {
    double acc = 0.0;
    for (int i = 0; i < KB; ++i) acc = fma(X[r][i], (double)T[i][t], acc);
    M[r * KB + t] = (float)acc;
  }
}

// dinv: [inv L blocks | inv U blocks | M of L | M of U], each ceil(n/64) x 4096.
cudaError_t diag_inverses(int n, const float* F, long long ldf, float* dinv, cudaStream_t s) {
  const int nblk = (n + 63) / 64;
  const size_t half = (size_t)nblk * 64 * 64;
  diag_inv_kernel<true><<<nblk, 64, 0, s>>>(n, F, ldf, dinv, dinv + 2 * half);
  diag_inv_kernel<false><<<nblk, 64, 0, s>>>(n, F, ldf, dinv + half, dinv + 3 * half);
  count_launches(2);
  return cudaGetLastError();
}

// Solve with the FP32 factors: Xf (n x nrhs, ld n) overwritten in place.
// Up to 8 right-hand sides use the single-launch chained solves.
static cudaError_t sgetrs_inplace(int n, int nrhs, const float* F, long long ldf, const int* perm,
                                  float* Xf, float* tmp, const MixedWork& mw, cudaStream_t s) {
  SL_TRY((permute_rows<float, float>(Xf, n, tmp, n, perm, n, nrhs, 0, s)));
  if (nrhs <= 8 && mw.chain && mw.epoch && mw.dinv) {
    const size_t half = (size_t)((n + 63) / 64) * 64 * 64;
    *mw.epoch += 1;
    SL_TRY((trsv_chain<float, float, true>(F, ldf, n, tmp, n, nrhs, mw.dinv, mw.dinv + 2 * half,
                                           mw.chain, *mw.epoch, mw.status, s)));
    *mw.epoch += 1;
    SL_TRY((trsv_chain<float, float, false>(F, ldf, n, tmp, n, nrhs, mw.dinv + half,
                                            mw.dinv + 3 * half, mw.chain, *mw.epoch, mw.status, s)));
  } else {
    SL_TRY(tri_solve<float>(true, false, true, n, nrhs, F, ldf, tmp, n, s));
    SL_TRY(tri_solve<float>(false, false, false, n, nrhs, F, ldf, tmp, n, s));
  }
  return cudaMemcpyAsync(Xf, tmp, sizeof(float) * (size_t)n * nrhs, cudaMemcpyDeviceToDevice, s);
}

// out = (LU)^-1 r in FP64 via the FP32 factors: r scaled per column by a power
// of two into FP32, solved, scaled back. beta = 0 overwrites, 1 accumulates.
static cudaError_t precond_apply(int n, int ncols, const double* r, long long ldr, double beta,
                                 double* out, long long ldo, const float* F, long long ldf,
                                 const MixedWork& mw, cudaStream_t s) {
  phase_begin(kPhPrecond, s);
  colmax_abs_kernel<<<ncols, 1024, 0, s>>>(r, ldr, n, mw.colmax);
  scale_to_float_kernel<<<blocks_for((long long)n * ncols), 256, 0, s>>>(r, ldr, n, ncols,
                                                                         mw.colmax, mw.Xf, n);
  count_launches(2);
  SL_TRY(sgetrs_inplace(n, ncols, F, ldf, mw.perm, mw.Xf, mw.Xtmp, mw, s));
  float_scaled_add_kernel<<<blocks_for((long long)n * ncols), 256, 0, s>>>(mw.Xf, n, n, ncols,
                                                                           mw.colmax, beta, out, ldo);
  count_launches(1);
  phase_end(kPhPrecond, s, 2.0 * (double)n * n * ncols, 4.0 * (double)n * n);
  return cudaGetLastError();
}

// out = (LU)^-1 r for one column with FP64 arithmetic on the FP32 factors
// (and their FP32 diagonal-block inverses): the preconditioner GMRES applies
// must be a fixed operator known to working precision, which an FP32 solve of
// a rounded right-hand side is not once kappa approaches 1/eps(FP32).
static cudaError_t precond_apply64(int n, const double* r, double* out, const float* F,
                                   long long ldf, const MixedWork& mw, cudaStream_t s) {
  if (!(mw.chain && mw.epoch && mw.dinv)) return precond_apply(n, 1, r, n, 0.0, out, n, F, ldf, mw, s);
  phase_begin(kPhPrecond, s);
  SL_TRY((permute_rows<double, double>(r, n, out, n, mw.perm, n, 1, 0, s)));
  const size_t half = (size_t)((n + 63) / 64) * 64 * 64;
  *mw.epoch += 1;
  SL_TRY((trsv_chain<float, double, true>(F, ldf, n, out, n, 1, mw.dinv, mw.dinv + 2 * half,
                                          mw.chain, *mw.epoch, mw.status, s)));
  *mw.epoch += 1;
  SL_TRY((trsv_chain<float, double, false>(F, ldf, n, out, n, 1, mw.dinv + half,
                                           mw.dinv + 3 * half, mw.chain, *mw.epoch, mw.status, s)));
  phase_end(kPhPrecond, s, 2.0 * (double)n * n, 4.0 * (double)n * n);
  return cudaSuccess;
}

// R = B - A X (FP64) for ncols columns.
static cudaError_t residual(int n, int ncols, const double* A, long long lda, const double* B,
                            long long ldb, const double* X, long long ldx, double* R,
                            cudaStream_t s) {
  phase_begin(kPhResidual, s);
  SL_TRY(cudaMemcpy2DAsync(R, n * sizeof(double), B, ldb * sizeof(double), n * sizeof(double),
                           ncols, cudaMemcpyDeviceToDevice, s));
  SL_TRY(gemm_update<double>(false, n, ncols, n, -1.0, A, lda, X, ldx, R, n, s));
  phase_end(kPhResidual, s, 2.0 * (double)n * n * ncols, 8.0 * (double)n * n);
  return cudaSuccess;
}

// Scaled residual per column (host): ||r||/(||A|| ||x|| n eps).
static cudaError_t scaled_residuals(int n, int ncols, const double* R, const double* X,
                                    long long ldx, double anorm, const MixedWork& mw,
                                    cudaStream_t s, std::vector<double>& out) {
  colmax_abs_kernel<<<ncols, 1024, 0, s>>>(R, n, n, mw.colmax);
  colmax_abs_kernel<<<ncols, 1024, 0, s>>>(X, ldx, n, mw.colmax + ncols);
  count_launches(2);
  std::vector<double> h(2 * (size_t)ncols);
  SL_TRY(cudaMemcpyAsync(h.data(), mw.colmax, sizeof(double) * 2 * ncols, cudaMemcpyDeviceToHost, s));
  SL_TRY(cudaStreamSynchronize(s));
  const double eps = std::ldexp(1.0, -53);
  out.resize(ncols);
  for (int c = 0; c < ncols; ++c) out[c] = h[c] / (h[ncols + c] * anorm * eps * n);
  return cudaSuccess;
}

// GMRES on (LU)^-1 A d = (LU)^-1 r for one column; d overwritten (starts 0).
// Returns the number of inner iterations in *its. From the fourth iteration
// on, the residual estimate's geometric rate (over the last four iterations
// from the eighth on, so that stagnation shows at once) predicts the
// iterations still needed to reach rtol; when those, at the iterations'
// measured host time, would take longer than budget_ms, the cycle stops and
// *gave_up is set (the caller then solves in FP64: refining on would cost
// more). budget_ms <= 0 turns the prediction off.
static cudaError_t gmres_column(int n, const double* A, long long lda, const double* r, double* d,
                                const float* F, long long ldf, const MixedWork& mw, int mmax,
                                double rtol, int* its, cudaStream_t s, double budget_ms,
                                bool* gave_up) {
  const auto t_start = std::chrono::steady_clock::now();
  double* V = mw.V;  // n x (mmax+1)
  const long long ldv = n;
  double* w = mw.w;
  std::vector<double> H((size_t)(mmax + 1) * mmax, 0.0), cs(mmax), sn(mmax), g(mmax + 1, 0.0);
  std::vector<double> hcol(mmax + 2);
  *its = 0;
  // v0 = M^-1 r / beta
  SL_TRY(precond_apply64(n, r, w, F, ldf, mw, s));
  dots_kernel<<<1, 1024, 0, s>>>(w, n, n, 1, w, mw.h);
  count_launches(1);
  double beta2 = 0.0;
  SL_TRY(cudaMemcpyAsync(&beta2, mw.h, sizeof(double), cudaMemcpyDeviceToHost, s));
  SL_TRY(cudaStreamSynchronize(s));
  const double beta = std::sqrt(beta2);
  SL_TRY(cudaMemsetAsync(d, 0, sizeof(double) * n, s));
  if (!(beta > 0.0) || !std::isfinite(beta)) return cudaSuccess;
  SL_TRY(cudaMemcpyAsync(mw.h + mmax + 4, &beta, sizeof(double), cudaMemcpyHostToDevice, s));
  scale_vec_kernel<<<blocks_for(n), 256, 0, s>>>(w, n, mw.h + mmax + 4, V);
  count_launches(1);
  g[0] = beta;
  int k = 0;
  for (; k < mmax; ++k) {
    // w = M^-1 A v_k
    phase_begin(kPhResidual, s);
    SL_TRY(cudaMemsetAsync(mw.Ax, 0, sizeof(double) * n, s));
    SL_TRY(gemm_update<double>(false, n, 1, n, 1.0, A, lda, V + (long long)k * ldv, ldv, mw.Ax, n, s));
    phase_end(kPhResidual, s, 2.0 * (double)n * n, 8.0 * (double)n * n);
    SL_TRY(precond_apply64(n, mw.Ax, w, F, ldf, mw, s));
    // classical Gram-Schmidt, twice
    std::fill(hcol.begin(), hcol.end(), 0.0);
    for (int pass = 0; pass < 2; ++pass) {
      dots_kernel<<<k + 1, 1024, 0, s>>>(V, ldv, n, k + 1, w, mw.h);
      sub_vh_kernel<<<blocks_for(n), 256, 0, s>>>(V, ldv, n, k + 1, mw.h, w);
      count_launches(2);
      std::vector<double> hp(k + 1);
      SL_TRY(cudaMemcpyAsync(hp.data(), mw.h, sizeof(double) * (k + 1), cudaMemcpyDeviceToHost, s));
      SL_TRY(cudaStreamSynchronize(s));
      for (int i = 0; i <= k; ++i) hcol[i] += hp[i];
    }
    dots_kernel<<<1, 1024, 0, s>>>(w, n, n, 1, w, mw.h);
    count_launches(1);
    double nw2 = 0.0;
    SL_TRY(cudaMemcpyAsync(&nw2, mw.h, sizeof(double), cudaMemcpyDeviceToHost, s));
    SL_TRY(cudaStreamSynchronize(s));
    const double hk1 = std::sqrt(nw2);
    hcol[k + 1] = hk1;
    if (hk1 > 0.0 && std::isfinite(hk1)) {
      SL_TRY(cudaMemcpyAsync(mw.h + mmax + 4, &hk1, sizeof(double), cudaMemcpyHostToDevice, s));
      scale_vec_kernel<<<blocks_for(n), 256, 0, s>>>(w, n, mw.h + mmax + 4, V + (long long)(k + 1) * ldv);
      count_launches(1);
    }
    // apply previous rotations, then a new one
    for (int i = 0; i < k; ++i) {
      double t = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
      hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
      hcol[i] = t;
    }
    const double a = hcol[k], b = hcol[k + 1];
    const double rr = std::hypot(a, b);
    cs[k] = rr > 0 ? a / rr : 1.0;
    sn[k] = rr > 0 ? b / rr : 0.0;
    hcol[k] = rr;
    hcol[k + 1] = 0.0;
    g[k + 1] = -sn[k] * g[k];
    g[k] = cs[k] * g[k];
    for (int i = 0; i <= k; ++i) H[(size_t)i + (size_t)k * (mmax + 1)] = hcol[i];
    *its = k + 1;
    if (std::fabs(g[k + 1]) <= rtol * beta || !(hk1 > 0.0)) { ++k; break; }
    if (k >= 3 && budget_ms > 0.0) {
      const double el = std::chrono::duration<double, std::milli>(
                            std::chrono::steady_clock::now() - t_start).count();
      const double gk = std::fabs(g[k + 1]);
      const double rate = k >= 7 ? std::pow(gk / std::fabs(g[k - 3]), 0.25)
                                 : std::pow(gk / beta, 1.0 / (double)(k + 1));
      const double need = (rate < 1.0 && gk > 0.0) ? std::log(rtol * beta / gk) / std::log(rate) : 1e30;
      if (need * el / (double)(k + 1) > budget_ms - el) { *gave_up = true; ++k; break; }
    }
  }
  // y = H(0:k,0:k)^-1 g ; d = V y
  std::vector<double> y(k, 0.0);
  for (int i = k - 1; i >= 0; --i) {
    double t = g[i];
    for (int j = i + 1; j < k; ++j) t -= H[(size_t)i + (size_t)j * (mmax + 1)] * y[j];
    const double hii = H[(size_t)i + (size_t)i * (mmax + 1)];
    y[i] = hii != 0.0 ? t / hii : 0.0;
  }
  if (k > 0) {
    SL_TRY(cudaMemcpyAsync(mw.h, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, s));
    add_vy_kernel<<<blocks_for(n), 256, 0, s>>>(V, ldv, n, k, mw.h, d);
    count_launches(1);
  }
  return cudaGetLastError();
}

cudaError_t dgesv_ir_device(int n, int nrhs, double* dA, long long lda, const double* dB,
                            long long ldb, double* dX, long long ldx, int* dipiv,
                            const IrOptions& opt, IrStats* st, const LuWork& ws,
                            const MixedWork& mw, cudaStream_t s) {
  *st = IrStats();
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  cudaEventRecord(e0, s);
  // ||A||_inf of the FP64 matrix (for the scaled residual)
  rowsum_abs_kernel<<<blocks_for(n), 256, 0, s>>>(dA, lda, n, mw.w);
  colmax_abs_kernel<<<1, 1024, 0, s>>>(mw.w, n, n, mw.colmax);
  count_launches(2);
  double anorm = 0.0;
  SL_TRY(cudaMemcpyAsync(&anorm, mw.colmax, sizeof(double), cudaMemcpyDeviceToHost, s));
  // FP32 working copy and low-precision factorization
  d2s_kernel<<<4 * num_sms(), 256, 0, s>>>(dA, lda, n, n, mw.F, mw.ldf);
  count_launches(1);
  SL_TRY(sgetrf_mixed_device(n, mw.F, mw.ldf, dipiv, opt.nb, opt.fmt, ws, mw, s));
  SL_TRY(perm_compose(dipiv, n, mw.perm, s));
  if (mw.dinv) SL_TRY(diag_inverses(n, mw.F, mw.ldf, mw.dinv, s));
  int hstat[2] = {0, 0};
  SL_TRY(cudaMemcpyAsync(hstat, ws.status, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  SL_TRY(cudaStreamSynchronize(s));
  cudaEventRecord(e1, s);
  // refinement budget: the estimated cost of the plain FP64 solve
  const auto t_ref0 = std::chrono::steady_clock::now();
  float fms = 0.f;
  SL_TRY(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&fms, e0, e1);
  const double budget_ms = opt.fp64_cost_ratio * (double)fms;
  auto budget_left = [&]() {
    if (!(budget_ms > 0.0)) return 0.0;  // rule off
    const double left = budget_ms - std::chrono::duration<double, std::milli>(
                                        std::chrono::steady_clock::now() - t_ref0).count();
    return left > 1e-3 ? left : 1e-3;
  };
  bool gave_up = false;
  st->anorm = anorm;
  bool ok_factor = (hstat[0] == 0) && !(hstat[1] >= 0 && hstat[1] < n);
  bool converged = false;
  std::vector<double> sres, prev;
  phase_begin(kPhRefine, s);
  if (ok_factor) {
    // x0 = (LU)^-1 b
    SL_TRY(precond_apply(n, nrhs, dB, ldb, 0.0, dX, ldx, mw.F, mw.ldf, mw, s));
    SL_TRY(residual(n, nrhs, dA, lda, dB, ldb, dX, ldx, mw.R, s));
    SL_TRY(scaled_residuals(n, nrhs, mw.R, dX, ldx, anorm, mw, s, sres));
    bool use_gmres = false;
    for (int it = 0; it < opt.max_ir; ++it) {
      double worst = *std::max_element(sres.begin(), sres.end());
      if (std::isfinite(worst) && worst <= opt.tol) { converged = true; break; }
      if (!prev.empty()) {
        double pw = *std::max_element(prev.begin(), prev.end());
        if (!(worst <= 0.5 * pw)) { use_gmres = true; break; }  // stalled
      }
      prev = sres;
      SL_TRY(precond_apply(n, nrhs, mw.R, n, 1.0, dX, ldx, mw.F, mw.ldf, mw, s));
      st->classical += 1;
      SL_TRY(residual(n, nrhs, dA, lda, dB, ldb, dX, ldx, mw.R, s));
      SL_TRY(scaled_residuals(n, nrhs, mw.R, dX, ldx, anorm, mw, s, sres));
    }
    if (!converged) {
      double worst = *std::max_element(sres.begin(), sres.end());
      converged = std::isfinite(worst) && worst <= opt.tol;
      if (!converged) use_gmres = true;
    }
    if (use_gmres && !converged) {
      prev.clear();
      for (int outer = 0; outer < opt.max_gmres_outer && !gave_up; ++outer) {
        double worst = *std::max_element(sres.begin(), sres.end());
        if (std::isfinite(worst) && worst <= opt.tol) { converged = true; break; }
        if (!prev.empty()) {
          double pw = *std::max_element(prev.begin(), prev.end());
          if (!(worst <= 0.9 * pw)) break;  // GMRES-IR stalled too
        }
        prev = sres;
        for (int c = 0; c < nrhs; ++c) {
          if (sres[c] <= opt.tol) continue;
          int its = 0;
          SL_TRY(gmres_column(n, dA, lda, mw.R + (long long)c * n, mw.D, mw.F, mw.ldf, mw,
                              opt.gmres_m, opt.gmres_rtol, &its, s, budget_left(), &gave_up));
          st->gmres_inner += its;
          axpy1_kernel<<<blocks_for(n), 256, 0, s>>>(n, mw.D, dX + (long long)c * ldx);  // x_c += d
          count_launches(1);
        }
        st->gmres_outer += 1;
        SL_TRY(residual(n, nrhs, dA, lda, dB, ldb, dX, ldx, mw.R, s));
        SL_TRY(scaled_residuals(n, nrhs, mw.R, dX, ldx, anorm, mw, s, sres));
      }
      if (!converged) {
        double worst = *std::max_element(sres.begin(), sres.end());
        converged = std::isfinite(worst) && worst <= opt.tol;
      }
    }
  }
  st->gave_up = (gave_up && !converged) ? 1 : 0;
  phase_end(kPhRefine, s, 0.0, 0.0);
  if (mw.status) {
    int cst = 0;
    SL_TRY(cudaMemcpyAsync(&cst, mw.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    SL_TRY(cudaStreamSynchronize(s));
    if (cst != 0) { st->dev_status = cst; return cudaSuccess; }
  }
  if (!converged) {
    // FP64 fallback with the plain FP64 path: on a copy of A when one was provided
    // (A preserved, the residual is reported), else in place as LAPACK DSGESV
    // does (A returns the FP64 factors).
    st->fell_back = 1;
    double* Af = dA;
    long long ldaf = lda;
    if (mw.Acopy) {
      SL_TRY(cudaMemcpy2DAsync(mw.Acopy, mw.ldacopy * sizeof(double), dA, lda * sizeof(double),
                               n * sizeof(double), n, cudaMemcpyDeviceToDevice, s));
      Af = mw.Acopy;
      ldaf = mw.ldacopy;
    }
    SL_TRY(dgetrf_device(n, n, Af, ldaf, dipiv, opt.nb_fp64, ws, s));
    SL_TRY(cudaMemcpyAsync(hstat, ws.status, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    SL_TRY(cudaStreamSynchronize(s));
    if (hstat[0] != 0) {
      st->dev_status = hstat[0];
    } else if (hstat[1] >= 0 && hstat[1] < n) {
      st->info = hstat[1] + 1;
    } else {
      SL_TRY(cudaMemcpy2DAsync(dX, ldx * sizeof(double), dB, ldb * sizeof(double),
                               n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s));
      SL_TRY(dgetrs_device('N', n, nrhs, Af, ldaf, dipiv, dX, ldx, ws, s));
      if (mw.Acopy) {
        SL_TRY(residual(n, nrhs, dA, lda, dB, ldb, dX, ldx, mw.R, s));
        SL_TRY(scaled_residuals(n, nrhs, mw.R, dX, ldx, anorm, mw, s, sres));
      } else {
        sres.assign(nrhs, -1.0);  // A was overwritten: the residual is not available here
      }
    }
  }
  cudaEventRecord(e2, s);
  SL_TRY(cudaEventSynchronize(e2));
  float t1 = 0.f, t2 = 0.f;
  cudaEventElapsedTime(&t1, e0, e1);
  cudaEventElapsedTime(&t2, e1, e2);
  st->factor_ms = t1;
  st->refine_ms = t2;
  st->sresid = sres.empty() ? -1.0 : *std::max_element(sres.begin(), sres.end());
  st->converged = converged ? 1 : 0;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  return cudaGetLastError();
}

}  // namespace sl
