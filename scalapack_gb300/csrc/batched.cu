// Batched solver: thousands of independent dense systems A_i X_i = B_i of
// uneven order (N_i <= 512) in one persistent launch. Each system is the same
// computation as PDGESV on a 1x1 grid (SRC/pdgesv.f: PDGETRF then PDGETRS),
// with LAPACK/ScaLAPACK pivoting semantics (first maximal |x|, scale by the
// reciprocal, INFO = first exactly-zero pivot).
//
// Layout: every system keeps its own column-major A_i (lda_i), B_i and X_i
// (ldb_i, ldx_i) in device memory; A_i and B_i are not modified. The plan
// holds a per-system workspace (a copy of A_i in the factorization precision)
// where the factors live, and the per-system outputs: pivots, INFO, refinement
// steps and the scaled residual ||b - A x||_inf / (||A||_inf ||x||_inf N eps).
//
// Scheduling: systems are sorted by decreasing N on the host (largest first,
// so the tail of the launch is made of small systems); CTAs of one persistent
// grid take the next system from an atomic ticket until the queue is empty.
//
// Per system, one CTA:
//   factor   blocked right-looking LU with 32-column panels held in shared
//            memory (IDAMAX by warp shuffles, swap, reciprocal scale, rank-1),
//            row interchanges on the other columns, U12 by forward
//            substitution from the shared L11, trailing update as a
//            register-tiled GEMM (each thread owns rows, CH columns at a time)
//   solve    composed permutation in shared memory, then 32-row blocked
//            forward / backward substitution (one warp per right-hand side
//            for the diagonal blocks, all threads for the off-diagonal update)
//   refine   (mode 1) FP32 factors, FP64 residual and update, at most kMaxIr
//            steps; a system that does not reach the tolerance is queued for
//            the FP64 pass, which is a second persistent launch in the same
//            CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <vector>

#include "common.cuh"
#include "sl_internal.h"

namespace sl {

constexpr int kBMaxN = 512;   // largest system order
constexpr int kBMaxRhs = 8;   // largest number of right-hand sides
constexpr int kBPB = 32;      // panel width
constexpr int kMaxIr = 10;    // refinement steps in mode 1

struct BatchArgs {
  int batch;
  const int* n;
  const int* nrhs;
  const double* const* A;
  const int* lda;
  const double* const* B;
  const int* ldb;
  double* const* X;
  const int* ldx;
  int* const* ipiv;
  void* const* W;        // per-system factor workspace (n x n in the factor type)
  void* const* W64;      // per-system FP64 workspace of the FP64 pass (== W in mode 0)
  const int* order;      // processing order (sorted by decreasing n)
  int* queue;            // [0] ticket of the main pass, [1] ticket of the fallback pass,
                         // [2] number of systems queued for the fallback pass
  int* fallback_list;    // systems queued for the FP64 pass
  int* info;
  int* iters;            // refinement steps; -1 = solved by the FP64 pass after refinement stalled
  double* sresid;
  double tol;
};

// ------------------------------------------------------------ helpers
template <typename T>
__device__ __forceinline__ void block_argmax(const T* P, int ldp, int k, int m, int& piv_out,
                                             double* s_key, int* s_row) {
  // IDAMAX over P[k..m-1][k]: first maximal |x|, NaN never wins except as the
  // first element (reference BLAS).
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  double key = -2.0;
  int row = 0x7fffffff;
  for (int r = k + tid; r < m; r += blockDim.x) amax_combine(key, row, amax_key((double)P[r * ldp + k]), r);
  warp_amax(key, row);
  if (lane == 0) { s_key[warp] = key; s_row[warp] = row; }
  __syncthreads();
  if (warp == 0) {
    key = lane < nw ? s_key[lane] : -2.0;
    row = lane < nw ? s_row[lane] : 0x7fffffff;
    warp_amax(key, row);
    if (lane == 0) {
      double d = (double)P[k * ldp + k];
      if (d != d || key == 0.0) row = k;
      s_row[0] = row;
    }
  }
  __syncthreads();
  piv_out = s_row[0];
}

// Factor the n x n matrix W (column-major, ld n) in place. ipiv receives
// 0-based rows; returns INFO (first zero pivot, 1-based) in *info.
// stage / stage_len: shared scratch idle during the factorization, used to
// apply each panel's row interchanges to the other columns.
template <typename T, int CH>
__device__ void factor_system(T* W, int n, int* ipiv, int* info, unsigned char* smem, T* stage,
                              int stage_len) {
  T* P = reinterpret_cast<T*>(smem);               // [kBMaxN][kBPB+1] panel, row-major
  T* Us = P + kBMaxN * (kBPB + 1);                   // [kBPB][CH+1] U12 chunk (padded rows)
  constexpr int UL = CH + 1;
  __shared__ double s_key[32];
  __shared__ int s_row[32];
  __shared__ int s_info;
  __shared__ int s_trow[2 * kBPB], s_tsrc[2 * kBPB], s_tcnt;
  const int tid = threadIdx.x, NT = blockDim.x;
  const int PL = kBPB + 1;
  if (tid == 0) s_info = 0;
  for (int j = 0; j < n; j += kBPB) {
    const int jb = min(kBPB, n - j);
    const int m = n - j;  // panel rows
    // load the panel rows j..n-1, columns j..j+jb-1
    for (int idx = tid; idx < m * jb; idx += NT) {
      int r = idx % m, c = idx / m;
      P[r * PL + c] = W[(j + r) + (long long)(j + c) * n];
    }
    __syncthreads();
    for (int k = 0; k < jb; ++k) {
      int piv;
      block_argmax<T>(P, PL, k, m, piv, s_key, s_row);
      if (tid == 0) ipiv[j + k] = j + piv;
      if (piv != k)
        for (int c = tid; c < jb; c += NT) {
          T t = P[k * PL + c];
          P[k * PL + c] = P[piv * PL + c];
          P[piv * PL + c] = t;
        }
      __syncthreads();
      const T g = P[k * PL + k];
      if (g == (T)0) {
        if (tid == 0 && s_info == 0) s_info = j + k + 1;
      }
      const T rinv = (g != (T)0) ? (T)1 / g : (T)0;
      for (int r = k + 1 + tid; r < m; r += NT) {
        T l = P[r * PL + k];
        if (g != (T)0) l *= rinv;
        P[r * PL + k] = l;
        for (int c = k + 1; c < jb; ++c) P[r * PL + c] = fma(-l, P[k * PL + c], P[r * PL + c]);
      }
      __syncthreads();
    }
    // write the panel back
    for (int idx = tid; idx < m * jb; idx += NT) {
      int r = idx % m, c = idx / m;
      W[(j + r) + (long long)(j + c) * n] = P[r * PL + c];
    }
    __syncthreads();
    // Row interchanges on the other columns (PDLASWP) as one composite
    // permutation: warp 0 replays the jb swaps on row labels (rows j..j+jb-1
    // and the pivot rows below), then every moved value of a chunk of
    // columns is read into `stage` before any is written back.
    if (tid < 32) {
      const int lane = tid;
      int cnt = jb;
      for (int e = lane; e < jb; e += 32) { s_trow[e] = j + e; s_tsrc[e] = j + e; }
      __syncwarp();
      for (int k = 0; k < jb; ++k) {
        const int p = ipiv[j + k];
        if (p == j + k) continue;
        int e = -1;
        if (p < j + jb) {
          e = p - j;
        } else {
          for (int base = jb; base < cnt && e < 0; base += 32) {
            const int q = base + lane;
            const unsigned hit = __ballot_sync(0xffffffffu, q < cnt && s_trow[q] == p);
            if (hit) e = base + __ffs(hit) - 1;
          }
          if (e < 0) {
            e = cnt++;
            if (lane == 0) { s_trow[e] = p; s_tsrc[e] = p; }
          }
        }
        __syncwarp();
        if (lane == 0) { const int t = s_tsrc[k]; s_tsrc[k] = s_tsrc[e]; s_tsrc[e] = t; }
        __syncwarp();
      }
      if (lane == 0) s_tcnt = cnt;
    }
    __syncthreads();
    {
      const int cnt = s_tcnt;
      const int cw = stage_len / cnt;  // columns per chunk (cnt <= 64)
      for (int c0 = 0; c0 < n; c0 += cw) {
        const int nc = min(cw, n - c0);
        for (int idx = tid; idx < nc * cnt; idx += NT) {
          const int e = idx % cnt, c = c0 + idx / cnt;
          if ((c < j || c >= j + jb) && s_tsrc[e] != s_trow[e])
            stage[idx] = W[s_tsrc[e] + (long long)c * n];
        }
        __syncthreads();
        for (int idx = tid; idx < nc * cnt; idx += NT) {
          const int e = idx % cnt, c = c0 + idx / cnt;
          if ((c < j || c >= j + jb) && s_tsrc[e] != s_trow[e])
            W[s_trow[e] + (long long)c * n] = stage[idx];
        }
        __syncthreads();
      }
    }
    const int nr = n - j - jb;  // trailing columns
    if (nr > 0) {
      // U12 = L11^-1 A12, one thread per column, L11 from the shared panel
      for (int c = j + jb + tid; c < n; c += NT) {
        T* col = W + (long long)c * n + j;
        T x[kBPB];
#pragma unroll
        for (int k = 0; k < kBPB; ++k) x[k] = k < jb ? col[k] : (T)0;
#pragma unroll
        for (int k = 0; k < kBPB; ++k)
#pragma unroll
          for (int r = k + 1; r < kBPB; ++r)
            if (r < jb) x[r] = fma(-P[r * PL + k], x[k], x[r]);
#pragma unroll
        for (int k = 0; k < kBPB; ++k)
          if (k < jb) col[k] = x[k];
      }
      __syncthreads();
      const int mr = m - jb;  // trailing rows
      if (mr > 0) {
        // A22 -= L21 * U12 in CH-column chunks: U12 chunk staged in shared memory,
        // each thread owns rows (coalesced column accesses) and CH accumulators.
        for (int c0 = j + jb; c0 < n; c0 += CH) {
          const int cw = min(CH, n - c0);
          for (int idx = tid; idx < jb * CH; idx += NT) {
            int k = idx % jb, c = idx / jb;
            Us[k * UL + c] = c < cw ? W[(j + k) + (long long)(c0 + c) * n] : (T)0;
          }
          __syncthreads();
          for (int r = tid; r < mr; r += NT) {
            T acc[CH];
#pragma unroll
            for (int c = 0; c < CH; ++c) acc[c] = (T)0;
            const T* lrow = P + (jb + r) * PL;
            for (int k = 0; k < jb; ++k) {
              const T a = lrow[k];
#pragma unroll
              for (int c = 0; c < CH; ++c) acc[c] = fma(a, Us[k * UL + c], acc[c]);
            }
            T* crow = W + (j + jb + r) + (long long)c0 * n;
#pragma unroll
            for (int c = 0; c < CH; ++c)
              if (c < cw) crow[(long long)c * n] -= acc[c];
          }
          __syncthreads();
        }
      }
    }
  }
  __syncthreads();
  if (tid == 0) *info = s_info;
  __syncthreads();
}

// The row permutation of the factorization (PDLAPIV's interchanges composed):
// perm[i] = original row that ends up in row i. Computed once per system.
__device__ void compose_perm(const int* ipiv, int n, int* perm) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = i;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int i = 0; i < n; ++i) {
      const int q = ipiv[i];
      if (q != i) { const int t = perm[i]; perm[i] = perm[q]; perm[q] = t; }
    }
  __syncthreads();
}

// Solve with the factors of factor_system: X (n x nrhs, ldx) holds the
// right-hand sides on entry and the solution on exit. Xs: shared scratch of
// n*nrhs values; perm: the composed permutation (shared memory).
template <typename T>
__device__ void solve_system(const T* W, int n, const int* perm, T* X, int ldx, int nrhs, T* Xs) {
  const int tid = threadIdx.x, NT = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int nw = NT >> 5;
  for (int idx = tid; idx < n * nrhs; idx += NT) {
    int i = idx % n, c = idx / n;
    Xs[i + c * n] = X[perm[i] + (long long)c * ldx];
  }
  __syncthreads();
  // forward (unit lower), 32-row blocks
  for (int k0 = 0; k0 < n; k0 += 32) {
    const int kb = min(32, n - k0);
    for (int c = warp; c < nrhs; c += nw) {
      T x = lane < kb ? Xs[k0 + lane + c * n] : (T)0;
      for (int i = 0; i < kb; ++i) {
        T xi = __shfl_sync(0xffffffffu, x, i);
        if (lane > i && lane < kb) x = fma(-W[(k0 + lane) + (long long)(k0 + i) * n], xi, x);
      }
      if (lane < kb) Xs[k0 + lane + c * n] = x;
    }
    __syncthreads();
    for (int r = k0 + kb + tid; r < n; r += NT) {
      T acc[kBMaxRhs];
#pragma unroll
      for (int c = 0; c < kBMaxRhs; ++c) acc[c] = (T)0;
      for (int i = 0; i < kb; ++i) {
        const T l = W[r + (long long)(k0 + i) * n];
#pragma unroll
        for (int c = 0; c < kBMaxRhs; ++c)
          if (c < nrhs) acc[c] = fma(l, Xs[k0 + i + c * n], acc[c]);
      }
#pragma unroll
      for (int c = 0; c < kBMaxRhs; ++c)
        if (c < nrhs) Xs[r + c * n] -= acc[c];
    }
    __syncthreads();
  }
  // backward (non-unit upper), 32-row blocks from the bottom
  const int nblk = (n + 31) / 32;
  for (int b = nblk - 1; b >= 0; --b) {
    const int k0 = b * 32;
    const int kb = min(32, n - k0);
    for (int c = warp; c < nrhs; c += nw) {
      T x = lane < kb ? Xs[k0 + lane + c * n] : (T)0;
      for (int i = kb - 1; i >= 0; --i) {
        if (lane == i) x = x / W[(k0 + i) + (long long)(k0 + i) * n];
        T xi = __shfl_sync(0xffffffffu, x, i);
        if (lane < i) x = fma(-W[(k0 + lane) + (long long)(k0 + i) * n], xi, x);
      }
      if (lane < kb) Xs[k0 + lane + c * n] = x;
    }
    __syncthreads();
    for (int r = tid; r < k0; r += NT) {
      T acc[kBMaxRhs];
#pragma unroll
      for (int c = 0; c < kBMaxRhs; ++c) acc[c] = (T)0;
      for (int i = 0; i < kb; ++i) {
        const T u = W[r + (long long)(k0 + i) * n];
#pragma unroll
        for (int c = 0; c < kBMaxRhs; ++c)
          if (c < nrhs) acc[c] = fma(u, Xs[k0 + i + c * n], acc[c]);
      }
#pragma unroll
      for (int c = 0; c < kBMaxRhs; ++c)
        if (c < nrhs) Xs[r + c * n] -= acc[c];
    }
    __syncthreads();
  }
  for (int idx = tid; idx < n * nrhs; idx += NT) {
    int i = idx % n, c = idx / n;
    X[i + (long long)c * ldx] = Xs[i + c * n];
  }
  __syncthreads();
}

// NaN-propagating maximum (a NaN, once seen, stays): the tester's norm semantics.
__device__ __forceinline__ double nanmax(double m, double v) { return (v > m || v != v) ? v : m; }

// R = B - A X (FP64) into shared Rs (n x nrhs); returns the scaled residual
// max_c ||r_c|| / (||A|| ||x_c|| n eps) (tester semantics, LIN/pdlaschk.f).
// X is staged in shared memory (Xsh, n*nrhs doubles) so the pass over A is the
// only global stream, read with 8 loads in flight per thread; ||A||_inf is
// passed in (*anorm >= 0, from the copy into the working matrix) or computed.
__device__ double residual_system(const double* A, int lda, int n, const double* B, int ldb,
                                  const double* X, int ldx, int nrhs, double* Rs, double* s_red,
                                  double* Xsh, double* anorm) {
  const int tid = threadIdx.x, NT = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int nw = NT >> 5;
  __shared__ double s_rm[32][kBMaxRhs], s_xm[32][kBMaxRhs];
  for (int idx = tid; idx < n * nrhs; idx += NT) {
    const int i = idx % n, c = idx / n;
    Xsh[i + c * n] = X[i + (long long)c * ldx];
  }
  __syncthreads();
  const bool need_norm = !(*anorm >= 0.0);
  double rowmax = 0.0;
  double rm[kBMaxRhs], xm[kBMaxRhs];
#pragma unroll
  for (int c = 0; c < kBMaxRhs; ++c) { rm[c] = 0.0; xm[c] = 0.0; }
  for (int r = tid; r < n; r += NT) {
    double acc[kBMaxRhs];
#pragma unroll
    for (int c = 0; c < kBMaxRhs; ++c) acc[c] = (c < nrhs) ? B[r + (long long)c * ldb] : 0.0;
    double rs = 0.0;
    const double* ar = A + r;
#pragma unroll 8
    for (int k = 0; k < n; ++k) {
      const double a = ar[(long long)k * lda];
      if (need_norm) rs += fabs(a);
#pragma unroll
      for (int c = 0; c < kBMaxRhs; ++c)
        if (c < nrhs) acc[c] = fma(-a, Xsh[k + c * n], acc[c]);
    }
    rowmax = fmax(rowmax, rs);
#pragma unroll
    for (int c = 0; c < kBMaxRhs; ++c)
      if (c < nrhs) {
        Rs[r + c * n] = acc[c];
        rm[c] = nanmax(rm[c], fabs(acc[c]));
        xm[c] = nanmax(xm[c], fabs(Xsh[r + c * n]));
      }
  }
  // block reductions: max row sum, and per column max |r| and max |x|
  for (int off = 16; off > 0; off >>= 1) {
    rowmax = fmax(rowmax, __shfl_xor_sync(0xffffffffu, rowmax, off));
#pragma unroll
    for (int c = 0; c < kBMaxRhs; ++c) {
      rm[c] = nanmax(rm[c], __shfl_xor_sync(0xffffffffu, rm[c], off));
      xm[c] = nanmax(xm[c], __shfl_xor_sync(0xffffffffu, xm[c], off));
    }
  }
  if (lane == 0) {
    s_red[warp] = rowmax;
#pragma unroll
    for (int c = 0; c < kBMaxRhs; ++c) { s_rm[warp][c] = rm[c]; s_xm[warp][c] = xm[c]; }
  }
  __syncthreads();
  if (tid == 0) {
    double an = *anorm;
    if (need_norm) {
      an = 0.0;
      for (int w = 0; w < nw; ++w) an = fmax(an, s_red[w]);
      *anorm = an;
    }
    double worst = 0.0;
    for (int c = 0; c < nrhs; ++c) {
      double r1 = 0.0, x1 = 0.0;
      for (int w = 0; w < nw; ++w) { r1 = nanmax(r1, s_rm[w][c]); x1 = nanmax(x1, s_xm[w][c]); }
      const double v = r1 / (x1 * an * ldexp(1.0, -53) * n);
      if (!(v <= worst)) worst = v;
    }
    s_red[32] = worst;
  }
  __syncthreads();
  return s_red[32];
}

template <typename TF, int CH>
__device__ void run_system(const BatchArgs& a, int sys, bool fp64_pass, unsigned char* smem) {
  const int n = a.n[sys], nrhs = a.nrhs[sys];
  const int tid = threadIdx.x, NT = blockDim.x;
  const double* A = a.A[sys];
  const int lda = a.lda[sys];
  TF* W = reinterpret_cast<TF*>(fp64_pass ? a.W64[sys] : a.W[sys]);
  int* ipiv = a.ipiv[sys];
  double* X = a.X[sys];
  const int ldx = a.ldx[sys];
  const double* B = a.B[sys];
  const int ldb = a.ldb[sys];
  // shared layout: factor scratch, then Xs (n*nrhs TF), Rs (n*nrhs double), perm (n ints)
  unsigned char* after = smem + sizeof(TF) * (kBMaxN * (kBPB + 1) + kBPB * (CH + 1));
  TF* Xs = reinterpret_cast<TF*>(after);
  double* Rs = reinterpret_cast<double*>(after + sizeof(double) * kBMaxN * kBMaxRhs);
  int* perm = reinterpret_cast<int*>(after + 2 * sizeof(double) * kBMaxN * kBMaxRhs);
  double* Xsh = reinterpret_cast<double*>(after);  // X staged by residual_system (Xs is idle then)
  __shared__ double s_red[40];
  __shared__ double s_anorm;
  __shared__ int s_info;
  __shared__ int s_ok;
  // working copy in the factorization precision; one thread per row, so the
  // same pass gives ||A||_inf (row sums of |a|)
  {
    double rs_max = 0.0;
    for (int r = tid; r < n; r += NT) {
      double rs = 0.0;
      const double* ar = A + r;
#pragma unroll 8
      for (int c = 0; c < n; ++c) {
        const double v = ar[(long long)c * lda];
        rs += fabs(v);
        W[r + (long long)c * n] = (TF)v;
      }
      rs_max = fmax(rs_max, rs);
    }
    for (int off = 16; off > 0; off >>= 1) rs_max = fmax(rs_max, __shfl_xor_sync(0xffffffffu, rs_max, off));
    if ((tid & 31) == 0) s_red[tid >> 5] = rs_max;
    __syncthreads();
    if (tid == 0) {
      double an = 0.0;
      for (int w = 0; w < (NT >> 5); ++w) an = fmax(an, s_red[w]);
      s_anorm = an;
    }
    __syncthreads();
  }
  // Xs and Rs are idle while factoring: they stage the row interchanges
  factor_system<TF, CH>(W, n, ipiv, &s_info, smem, reinterpret_cast<TF*>(after),
                        (int)(2 * sizeof(double) * kBMaxN * kBMaxRhs / sizeof(TF)));
  const int info = s_info;
  if (info != 0) {
    // Exactly singular in the factorization precision: in mode 1 hand the
    // system to the FP64 pass, else report INFO and leave X untouched.
    if (!fp64_pass && sizeof(TF) == 4) {
      if (tid == 0) {
        int slot = atomicAdd(&a.queue[2], 1);
        a.fallback_list[slot] = sys;
      }
    } else if (tid == 0) {
      a.info[sys] = info;
      a.iters[sys] = 0;
      a.sresid[sys] = -1.0;
    }
    __syncthreads();
    return;
  }
  compose_perm(ipiv, n, perm);
  if constexpr (sizeof(TF) == 8) {
    // FP64: X = B, solve, residual
    for (int idx = tid; idx < n * nrhs; idx += NT) {
      int i = idx % n, c = idx / n;
      X[i + (long long)c * ldx] = B[i + (long long)c * ldb];
    }
    __syncthreads();
    solve_system<TF>(W, n, perm, reinterpret_cast<TF*>(X), ldx, nrhs, Xs);
    double sr = residual_system(A, lda, n, B, ldb, X, ldx, nrhs, Rs, s_red, Xsh, &s_anorm);
    if (tid == 0) {
      a.info[sys] = 0;
      a.iters[sys] = fp64_pass ? -1 : 0;
      a.sresid[sys] = sr;
    }
    __syncthreads();
    return;
  } else {
    // FP32 factors + FP64 refinement.
    for (int idx = tid; idx < n * nrhs; idx += NT) {
      int i = idx % n, c = idx / n;
      X[i + (long long)c * ldx] = 0.0;
    }
    __syncthreads();
    // initial residual r = b (x = 0): no pass over A
    for (int idx = tid; idx < n * nrhs; idx += NT) {
      const int i = idx % n, c = idx / n;
      Rs[i + c * n] = B[i + (long long)c * ldb];
    }
    __syncthreads();
    double sr = 1.0 / 0.0;  // scaled residual of x = 0 (the loop always refines at least once)
    int steps = 0;
    if (tid == 0) s_ok = 0;
    __syncthreads();
    for (int it = 0; it <= kMaxIr; ++it) {
      if (it > 0 && sr <= a.tol) { if (tid == 0) s_ok = 1; break; }
      if (it == kMaxIr) break;
      // correction: scale each residual column by a power of two into FP32, solve
      __shared__ int s_exp[kBMaxRhs];
      if (tid < nrhs) {
        double mx = 0.0;
        for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(Rs[i + tid * n]));
        int e = 0;
        if (mx > 0.0 && isfinite(mx)) frexp(mx, &e);
        s_exp[tid] = e;
      }
      __syncthreads();
      // copy the scaled residual into an FP32 buffer laid out like X (ld = n)
      TF* Cx = Xs + n * nrhs;  // second half of the Xs region (n*nrhs <= 4096 floats)
      for (int idx = tid; idx < n * nrhs; idx += NT) {
        int i = idx % n, c = idx / n;
        Cx[i + c * n] = (TF)ldexp(Rs[i + c * n], -s_exp[c]);
      }
      __syncthreads();
      solve_system<TF>(W, n, perm, Cx, n, nrhs, Xs);
      for (int idx = tid; idx < n * nrhs; idx += NT) {
        int i = idx % n, c = idx / n;
        X[i + (long long)c * ldx] += ldexp((double)Cx[i + c * n], s_exp[c]);
      }
      __syncthreads();
      ++steps;
      sr = residual_system(A, lda, n, B, ldb, X, ldx, nrhs, Rs, s_red, Xsh, &s_anorm);
    }
    if (s_ok) {
      if (tid == 0) {
        a.info[sys] = 0;
        a.iters[sys] = steps;
        a.sresid[sys] = sr;
      }
    } else if (tid == 0) {
      int slot = atomicAdd(&a.queue[2], 1);
      a.fallback_list[slot] = sys;
    }
    __syncthreads();
  }
}

template <typename TF, int CH>
__global__ void batched_kernel(BatchArgs a, int fp64_pass) {
  extern __shared__ __align__(16) unsigned char bsmem[];
  __shared__ int s_item;
  const int ticket = fp64_pass ? 1 : 0;
  const int count = fp64_pass ? a.queue[2] : a.batch;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(&a.queue[ticket], 1);
    __syncthreads();
    const int item = s_item;
    if (item >= count) break;
    const int sys = fp64_pass ? a.fallback_list[item] : a.order[item];
    run_system<TF, CH>(a, sys, fp64_pass != 0, bsmem);
  }
}

template <typename TF, int CH>
size_t batched_smem() {
  return sizeof(TF) * (kBMaxN * (kBPB + 1) + kBPB * (CH + 1)) + 2 * sizeof(double) * kBMaxN * kBMaxRhs +
         sizeof(int) * kBMaxN + 64;
}

template <typename TF, int CH>
cudaError_t launch_batched(const BatchArgs& a, int fp64_pass, int threads, int ctas_per_sm,
                           cudaStream_t s) {
  const size_t smem = batched_smem<TF, CH>();
  auto kern = batched_kernel<TF, CH>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  int occ = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, threads, smem);
  if (e != cudaSuccess) return e;
  if (occ < 1) return cudaErrorInvalidConfiguration;
  const int per_sm = std::min(occ, std::max(1, ctas_per_sm));
  kern<<<num_sms() * per_sm, threads, smem, s>>>(a, fp64_pass);
  count_launches(1);
  return cudaGetLastError();
}

// ------------------------------------------------------------ plan
struct BatchPlan {
  int batch = 0, mode = 0;
  double tol = 1.0;
  // device arrays
  int *d_n = nullptr, *d_nrhs = nullptr, *d_lda = nullptr, *d_ldb = nullptr, *d_ldx = nullptr;
  const double** d_A = nullptr;
  const double** d_B = nullptr;
  double** d_X = nullptr;
  int** d_ipiv = nullptr;
  void** d_W = nullptr;
  int *d_order = nullptr, *d_queue = nullptr, *d_fb = nullptr;
  int *d_info = nullptr, *d_iters = nullptr;
  double* d_sresid = nullptr;
  void* work = nullptr;        // factor workspaces (one block)
  void* work64 = nullptr;      // FP64 workspaces of the FP64 pass (mode 1)
  void** d_W64 = nullptr;
  int* ipiv_pool = nullptr;    // pivots (one block)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int threads = 256, chunk = 32, ctas_per_sm = 1;
  double flops = 0.0;
};

static BatchArgs plan_args(const BatchPlan& p) {
  BatchArgs a;
  a.batch = p.batch; a.n = p.d_n; a.nrhs = p.d_nrhs; a.A = p.d_A; a.lda = p.d_lda;
  a.B = p.d_B; a.ldb = p.d_ldb; a.X = p.d_X; a.ldx = p.d_ldx; a.ipiv = p.d_ipiv; a.W = p.d_W;
  a.W64 = p.mode == 0 ? p.d_W : p.d_W64;
  a.order = p.d_order; a.queue = p.d_queue; a.fallback_list = p.d_fb; a.info = p.d_info;
  a.iters = p.d_iters; a.sresid = p.d_sresid; a.tol = p.tol;
  return a;
}

static cudaError_t record_plan(const BatchPlan& p, int threads, int chunk, int ctas, cudaStream_t s) {
  BatchArgs a = plan_args(p);
  SL_TRY(cudaMemsetAsync(p.d_queue, 0, 4 * sizeof(int), s));
  if (p.mode == 0) {
    if (chunk == 64) return launch_batched<double, 64>(a, 0, threads, ctas, s);
    return launch_batched<double, 32>(a, 0, threads, ctas, s);
  }
  if (chunk == 64) SL_TRY((launch_batched<float, 64>(a, 0, threads, ctas, s)));
  else SL_TRY((launch_batched<float, 32>(a, 0, threads, ctas, s)));
  // FP64 pass over the systems the refinement could not finish (may be empty)
  return launch_batched<double, 32>(a, 1, 256, 1, s);
}

cudaError_t batch_plan_create(BatchPlan** out, int batch, const int* n, const int* nrhs,
                              const double* const* A, const int* lda, const double* const* B,
                              const int* ldb, double* const* X, const int* ldx, int mode,
                              double tol, int autotune, cudaStream_t s) {
  *out = nullptr;
  BatchPlan* p = new BatchPlan();
  p->batch = batch;
  p->mode = mode;
  p->tol = tol > 0 ? tol : 1.0;
  std::vector<int> order(batch);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return n[x] > n[y]; });
  const size_t esz = mode == 0 ? sizeof(double) : sizeof(float);
  std::vector<size_t> woff(batch), poff(batch);
  size_t wtot = 0, ptot = 0;
  for (int i = 0; i < batch; ++i) {
    woff[i] = wtot;
    wtot += ((size_t)n[i] * n[i] * esz + 255) / 256 * 256;
    poff[i] = ptot;
    ptot += (size_t)n[i];
    p->flops += 2.0 * n[i] * (double)n[i] * n[i] / 3.0;
  }
  cudaError_t e = cudaSuccess;
  auto alloc = [&](auto** ptr, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc((void**)ptr, bytes < 4 ? 4 : bytes);
  };
  alloc(&p->d_n, sizeof(int) * batch);
  alloc(&p->d_nrhs, sizeof(int) * batch);
  alloc(&p->d_lda, sizeof(int) * batch);
  alloc(&p->d_ldb, sizeof(int) * batch);
  alloc(&p->d_ldx, sizeof(int) * batch);
  alloc(&p->d_A, sizeof(double*) * batch);
  alloc(&p->d_B, sizeof(double*) * batch);
  alloc(&p->d_X, sizeof(double*) * batch);
  alloc(&p->d_ipiv, sizeof(int*) * batch);
  alloc(&p->d_W, sizeof(void*) * batch);
  alloc(&p->d_order, sizeof(int) * batch);
  alloc(&p->d_queue, sizeof(int) * 4);
  alloc(&p->d_fb, sizeof(int) * batch);
  alloc(&p->d_info, sizeof(int) * batch);
  alloc(&p->d_iters, sizeof(int) * batch);
  alloc(&p->d_sresid, sizeof(double) * batch);
  alloc(&p->work, wtot);
  alloc(&p->ipiv_pool, sizeof(int) * ptot);
  std::vector<size_t> w64off(batch);
  size_t w64 = 0;
  if (mode == 1) {
    for (int i = 0; i < batch; ++i) {
      w64off[i] = w64;
      w64 += ((size_t)n[i] * n[i] * sizeof(double) + 255) / 256 * 256;
    }
    alloc(&p->work64, w64);
    alloc(&p->d_W64, sizeof(void*) * batch);
  }
  if (e != cudaSuccess) { batch_plan_destroy(p); return e; }
  std::vector<void*> W(batch), W64(batch);
  std::vector<int*> piv(batch);
  for (int i = 0; i < batch; ++i) {
    W[i] = (unsigned char*)p->work + woff[i];
    if (mode == 1) W64[i] = (unsigned char*)p->work64 + w64off[i];
    piv[i] = p->ipiv_pool + poff[i];
  }
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  };
  up(p->d_n, n, sizeof(int) * batch);
  up(p->d_nrhs, nrhs, sizeof(int) * batch);
  up(p->d_lda, lda, sizeof(int) * batch);
  up(p->d_ldb, ldb, sizeof(int) * batch);
  up(p->d_ldx, ldx, sizeof(int) * batch);
  up(p->d_A, A, sizeof(double*) * batch);
  up(p->d_B, B, sizeof(double*) * batch);
  up(p->d_X, X, sizeof(double*) * batch);
  up(p->d_ipiv, piv.data(), sizeof(int*) * batch);
  up(p->d_W, W.data(), sizeof(void*) * batch);
  if (mode == 1) up(p->d_W64, W64.data(), sizeof(void*) * batch);
  up(p->d_order, order.data(), sizeof(int) * batch);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { batch_plan_destroy(p); return e; }
  // autotune: time the candidate shapes on this batch and keep the fastest
  struct Cand { int threads, chunk, ctas; };
  std::vector<Cand> cands = {{256, 32, 1}, {256, 64, 1}, {512, 32, 1}, {128, 32, 2}};
  Cand best = cands[0];
  if (autotune) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best_ms = 1e30f;
    for (const Cand& c : cands) {
      cudaEventRecord(e0, s);
      cudaError_t r = record_plan(*p, c.threads, c.chunk, c.ctas, s);
      cudaEventRecord(e1, s);
      if (r != cudaSuccess) { cudaGetLastError(); continue; }
      if (cudaEventSynchronize(e1) != cudaSuccess) break;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best_ms) { best_ms = ms; best = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  p->threads = best.threads;
  p->chunk = best.chunk;
  p->ctas_per_sm = best.ctas;
  // capture the execution in a CUDA graph
  cudaStream_t cs;
  e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t r = record_plan(*p, p->threads, p->chunk, p->ctas_per_sm, cs);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(cs, &g);
    if (r != cudaSuccess) e = r;
    if (e == cudaSuccess) {
      p->graph = g;
      e = cudaGraphInstantiate(&p->exec, g, 0);
    }
  }
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) { batch_plan_destroy(p); return e; }
  *out = p;
  return cudaSuccess;
}

cudaError_t batch_plan_execute(BatchPlan* p, cudaStream_t s) {
  phase_begin(kPhBatched, s);
  cudaError_t e = cudaGraphLaunch(p->exec, s);
  count_launches(p->mode == 0 ? 1 : 2);
  phase_end(kPhBatched, s, p->flops, 0.0);
  return e;
}

cudaError_t batch_plan_results(BatchPlan* p, int* info, int* iters, double* sresid,
                               cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  if (info) e = cudaMemcpyAsync(info, p->d_info, sizeof(int) * p->batch, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && iters)
    e = cudaMemcpyAsync(iters, p->d_iters, sizeof(int) * p->batch, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && sresid)
    e = cudaMemcpyAsync(sresid, p->d_sresid, sizeof(double) * p->batch, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

void batch_plan_shape(const BatchPlan* p, int* threads, int* chunk, int* ctas) {
  *threads = p->threads;
  *chunk = p->chunk;
  *ctas = p->ctas_per_sm;
}

void batch_plan_destroy(BatchPlan* p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  cudaFree(p->d_n); cudaFree(p->d_nrhs); cudaFree(p->d_lda); cudaFree(p->d_ldb); cudaFree(p->d_ldx);
  cudaFree(p->d_A); cudaFree(p->d_B); cudaFree(p->d_X); cudaFree(p->d_ipiv); cudaFree(p->d_W);
  cudaFree(p->d_order); cudaFree(p->d_queue); cudaFree(p->d_fb); cudaFree(p->d_info);
  cudaFree(p->d_iters); cudaFree(p->d_sresid); cudaFree(p->work); cudaFree(p->ipiv_pool);
  cudaFree(p->work64); cudaFree(p->d_W64);
  delete p;
}

}  // namespace sl
