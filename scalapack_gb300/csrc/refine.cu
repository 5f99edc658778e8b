// Iterative refinement with error bounds and equilibration on the GPU:
//
//   dgerfs_device  PDGERFS (SRC/pdgerfs.f:470-887): per right-hand side, the
//                  FP64 residual r = b - op(A) x and w = |b| + |op(A)| |x| in
//                  one pass over A, the componentwise backward error
//                  BERR = max_i |r_i| / w_i, refinement steps
//                  x += op(AF)^-1 r while BERR > eps, halves, and at most 5
//                  steps were taken (ITMAX = 5), and the forward error bound
//                  FERR = ||inv(op(A)) diag(|r| + nz eps w)||_inf / ||x||_inf
//                  with the PDLACON estimator;
//   dgeequ_device  PDGEEQU (SRC/pdgeequ.f): row and column scale factors;
//   dlaqge_device  PDLAQGE (SRC/pdlaqge.f): applies them when worthwhile.
//
// Layout: every vector is a contiguous FP64 array in HBM; A and AF are
// column-major with their own leading dimensions. The residual kernel for
// op = N splits the columns over CTAs (partials summed in a fixed order, so
// results are deterministic); for op = T one CTA reduces each column.
#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <cmath>

#include "common.cuh"
#include "sl_internal.h"

namespace sl {

__global__ void iamax_kernel(const double* __restrict__ z, int n, int* jout, double* vout);

namespace {

constexpr int kMaxSplit = 16;

// Row strip of 256 rows x one column slice: partial sums of a_ij x_j and
// |a_ij| |x_j| (op = N).
__global__ void __launch_bounds__(256)
resid_abs_n_part_kernel(int n, const double* __restrict__ A, long long lda,
                        const double* __restrict__ x, int kslice, double* part) {
  __shared__ double xs[256];
  const long long row = (long long)blockIdx.x * 256 + threadIdx.x;
  const int k0 = blockIdx.y * kslice;
  const int k1 = min(n, k0 + kslice);
  double s = 0.0, t = 0.0;
  for (int kc = k0; kc < k1; kc += 256) {
    const int kn = min(256, k1 - kc);
    __syncthreads();
    if ((int)threadIdx.x < kn) xs[threadIdx.x] = x[kc + threadIdx.x];
    __syncthreads();
    if (row < n) {
      const double* a = A + row + (long long)kc * lda;
#pragma unroll 8
      for (int kk = 0; kk < kn; ++kk) {
        const double v = a[(long long)kk * lda];
        s = fma(v, xs[kk], s);
        t = fma(fabs(v), fabs(xs[kk]), t);
      }
    }
  }
  if (row < n) {
    part[((size_t)blockIdx.y * 2 + 0) * n + row] = s;
    part[((size_t)blockIdx.y * 2 + 1) * n + row] = t;
  }
}

__global__ void resid_abs_n_reduce_kernel(int n, int ks, const double* __restrict__ part,
                                          const double* __restrict__ b, double* r, double* w) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0, t = 0.0;
  for (int k = 0; k < ks; ++k) {
    s += part[((size_t)k * 2 + 0) * n + i];
    t += part[((size_t)k * 2 + 1) * n + i];
  }
  r[i] = b[i] - s;
  w[i] = fabs(b[i]) + t;
}

// op = T: CTA j reduces column j of A against x.
__global__ void __launch_bounds__(256)
resid_abs_t_kernel(int n, const double* __restrict__ A, long long lda, const double* __restrict__ x,
                   const double* __restrict__ b, double* r, double* w) {
  __shared__ double ss[8], st[8];
  const int j = blockIdx.x;
  const double* a = A + (long long)j * lda;
  double s = 0.0, t = 0.0;
  for (int i = threadIdx.x; i < n; i += 256) {
    const double v = a[i];
    s = fma(v, x[i], s);
    t = fma(fabs(v), fabs(x[i]), t);
  }
  for (int off = 16; off > 0; off >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, off);
    t += __shfl_xor_sync(0xffffffffu, t, off);
  }
  if ((threadIdx.x & 31) == 0) { ss[threadIdx.x >> 5] = s; st[threadIdx.x >> 5] = t; }
  __syncthreads();
  if (threadIdx.x == 0) {
    s = 0.0;
    t = 0.0;
    for (int q = 0; q < 8; ++q) { s += ss[q]; t += st[q]; }
    r[j] = b[j] - s;
    w[j] = fabs(b[j]) + t;
  }
}

// BERR = max_i |r_i| / w_i, with SAFE1 added to both when w_i <= SAFE2
// (SRC/pdgerfs.f:588-603).
__global__ void berr_kernel(int n, const double* __restrict__ r, const double* __restrict__ w,
                            double safe1, double safe2, double* out) {
  __shared__ double sm[32];
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double q = (w[i] > safe2) ? fabs(r[i]) / w[i] : (fabs(r[i]) + safe1) / (w[i] + safe1);
    m = fmax(m, q);
  }
  for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    if (threadIdx.x == 0) *out = m;
  }
}

// w_i = |r_i| + nz eps w_i (+ SAFE1 when w_i <= SAFE2) (SRC/pdgerfs.f:646-656).
__global__ void ferr_weight_kernel(int n, const double* __restrict__ r, double* w, double nzeps,
                                   double safe1, double safe2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double wi = w[i];
  w[i] = (wi > safe2) ? fabs(r[i]) + nzeps * wi : fabs(r[i]) + nzeps * wi + safe1;
}

__global__ void vmul_kernel(int n, double* x, const double* __restrict__ w) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = w[i] * x[i];
}

__global__ void axpy1_kernel(int n, const double* __restrict__ d, double* x) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = x[i] + d[i];
}

// ---- equilibration -------------------------------------------------------

// rmax[i] (as ordered bits of a non-negative double) = max_j |a_ij| over one
// column slice per CTA row; maxima are exact, so the atomic order is irrelevant.
__global__ void __launch_bounds__(256)
rowmax_abs_kernel(int m, int n, const double* __restrict__ A, long long lda, int kslice,
                  unsigned long long* rmax) {
  const long long row = (long long)blockIdx.x * 256 + threadIdx.x;
  if (row >= m) return;
  const int k0 = blockIdx.y * kslice, k1 = min(n, k0 + kslice);
  double mx = 0.0;
  const double* a = A + row;
#pragma unroll 8
  for (int j = k0; j < k1; ++j) mx = fmax(mx, fabs(a[(long long)j * lda]));
  atomicMax(rmax + row, (unsigned long long)__double_as_longlong(mx));
}

// c[j] = max_i |a_ij| * r_i (SRC/pdgeequ.f, loop 90).
__global__ void __launch_bounds__(256)
colmax_scaled_kernel(int m, const double* __restrict__ A, long long lda,
                     const double* __restrict__ r, double* c) {
  __shared__ double sm[8];
  const int j = blockIdx.x;
  const double* a = A + (long long)j * lda;
  double mx = 0.0;
  for (int i = threadIdx.x; i < m; i += 256) mx = fmax(mx, fabs(a[i]) * r[i]);
  for (int off = 16; off > 0; off >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < 8; ++q) mx = fmax(mx, sm[q]);
    mx = fmax(mx, sm[0]);
    c[j] = mx;
  }
}

// out[0] = max v, out[1] = min v, *first0 = 1 + first index with v == 0 (0 if none).
__global__ void minmax_kernel(int k, const double* __restrict__ v, double init_min, double* out,
                              int* first0) {
  __shared__ double smx[32], smn[32];
  __shared__ int sz[32];
  double mx = 0.0, mn = init_min;
  int z = INT_MAX;
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const double x = v[i];
    mx = fmax(mx, x);
    mn = fmin(mn, x);
    if (x == 0.0 && i < z) z = i;
  }
  for (int off = 16; off > 0; off >>= 1) {
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, off));
    z = min(z, __shfl_xor_sync(0xffffffffu, z, off));
  }
  if ((threadIdx.x & 31) == 0) { smx[threadIdx.x >> 5] = mx; smn[threadIdx.x >> 5] = mn; sz[threadIdx.x >> 5] = z; }
  __syncthreads();
  if (threadIdx.x < 32) {
    const bool live = threadIdx.x < (blockDim.x >> 5);
    mx = live ? smx[threadIdx.x] : 0.0;
    mn = live ? smn[threadIdx.x] : init_min;
    z = live ? sz[threadIdx.x] : INT_MAX;
    for (int off = 16; off > 0; off >>= 1) {
      mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, off));
      mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, off));
      z = min(z, __shfl_xor_sync(0xffffffffu, z, off));
    }
    if (threadIdx.x == 0) {
      out[0] = mx;
      out[1] = mn;
      *first0 = (z == INT_MAX) ? 0 : z + 1;
    }
  }
}

// v_i = 1 / min(max(v_i, smlnum), bignum) (SRC/pdgeequ.f, loops 60 and 120).
__global__ void recip_clamp_kernel(int k, double* v, double smlnum, double bignum) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) v[i] = 1.0 / fmin(fmax(v[i], smlnum), bignum);
}

__global__ void bits_to_double_kernel(int k, const unsigned long long* __restrict__ b, double* v) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) v[i] = __longlong_as_double((long long)b[i]);
}

// A := diag(R) A diag(C) in the form EQUED names (SRC/pdlaqge.f): 'C' c_j a_ij,
// 'R' r_i a_ij, 'B' (c_j r_i) a_ij.
__global__ void laqge_kernel(int m, int n, double* A, long long lda, const double* __restrict__ r,
                             const double* __restrict__ c, int mode) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)m * n) return;
  const long long i = idx % m, j = idx / m;
  double& a = A[i + j * lda];
  if (mode == 'C') a = c[j] * a;
  else if (mode == 'R') a = r[i] * a;
  else a = c[j] * r[i] * a;
}

// X(i, c) = v_i X(i, c) for c < ncols.
__global__ void scale_rows_kernel(int n, int ncols, double* X, long long ldx,
                                  const double* __restrict__ v) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * ncols) return;
  const long long i = idx % n, c = idx / n;
  X[i + c * ldx] = v[i] * X[i + c * ldx];
}

unsigned blocks(long long k, int t = 256) { return (unsigned)((k + t - 1) / t); }

cudaError_t read_sync(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  SL_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s));
  return cudaStreamSynchronize(s);
}

}  // namespace

size_t refine_work_doubles(int n) {
  const size_t nn = (size_t)(n > 0 ? n : 1);
  return 2 * nn + (3 * nn + 4) + 2 * (size_t)kMaxSplit * nn + 16;
}

cudaError_t dgerfs_device(char trans, int n, int nrhs, const double* A, long long lda,
                          const double* AF, long long ldaf, const int* dipiv, const double* B,
                          long long ldb, double* X, long long ldx, double* ferr, double* berr,
                          const LuWork& ws, double* work, int* iw, cudaStream_t s) {
  const bool notran = (trans == 'N');
  const char transt = notran ? 'T' : 'N';
  if (n <= 1 || nrhs == 0) {
    for (int k = 0; k < nrhs; ++k) { ferr[k] = 0.0; berr[k] = 0.0; }
    return cudaSuccess;
  }
  double* r = work;
  double* w = work + n;
  double* lw = work + 2 * (size_t)n;                 // estimator workspace (3n + 4)
  double* part = lw + 3 * (size_t)n + 4;              // split-K partials
  double* scal = part + 2 * (size_t)kMaxSplit * n;    // scalars
  // NZ = N + 1; EPS = 2^-53 and SAFMIN = 2^-1022 (PDLAMCH 'Epsilon', 'Safe minimum')
  const int nz = n + 1;
  const double eps = DBL_EPSILON * 0.5;
  const double safmin = DBL_MIN;
  const double safe1 = nz * safmin;
  const double safe2 = safe1 / eps;
  const int rb = (n + 255) / 256;
  int ks = (4 * num_sms() + rb - 1) / rb;
  if (ks < 1) ks = 1;
  if (ks > kMaxSplit) ks = kMaxSplit;
  const int kslice = (n + ks - 1) / ks;
  ks = (n + kslice - 1) / kslice;
  const unsigned g = blocks(n);

  auto residual = [&](const double* x, const double* b) -> cudaError_t {
    if (notran) {
      resid_abs_n_part_kernel<<<dim3(rb, ks), 256, 0, s>>>(n, A, lda, x, kslice, part);
      resid_abs_n_reduce_kernel<<<g, 256, 0, s>>>(n, ks, part, b, r, w);
      count_launches(2);
    } else {
      resid_abs_t_kernel<<<n, 256, 0, s>>>(n, A, lda, x, b, r, w);
      count_launches(1);
    }
    return cudaGetLastError();
  };

  for (int k = 0; k < nrhs; ++k) {
    double* x = X + (long long)k * ldx;
    const double* b = B + (long long)k * ldb;
    int count = 1;
    double lstres = 3.0;
    double sres = 0.0;
    for (;;) {
      SL_TRY(residual(x, b));
      berr_kernel<<<1, 1024, 0, s>>>(n, r, w, safe1, safe2, scal);
      count_launches(1);
      SL_TRY(cudaGetLastError());
      SL_TRY(read_sync(&sres, scal, sizeof(double), s));
      berr[k] = sres;
      // continue while BERR > eps, it at least halved, and ITMAX = 5 steps
      if (sres > eps && 2.0 * sres <= lstres && count <= 5) {
        SL_TRY(dgetrs_device(trans, n, 1, AF, ldaf, dipiv, r, n, ws, s));
        axpy1_kernel<<<g, 256, 0, s>>>(n, r, x);
        count_launches(1);
        lstres = sres;
        ++count;
        continue;
      }
      break;
    }
    // FERR: ||inv(op(A)) diag(W)||_inf with W = |r| + nz eps (|op(A)||x| + |b|)
    ferr_weight_kernel<<<g, 256, 0, s>>>(n, r, w, (double)nz * eps, safe1, safe2);
    count_launches(1);
    double est = 0.0;
    SL_TRY(lacon_estimate(
        n,
        [&](bool kase1, double* v) -> cudaError_t {
          if (kase1) {  // diag(W) inv(op(A))^T
            SL_TRY(dgetrs_device(transt, n, 1, AF, ldaf, dipiv, v, n, ws, s));
            vmul_kernel<<<g, 256, 0, s>>>(n, v, w);
          } else {      // inv(op(A)) diag(W)
            vmul_kernel<<<g, 256, 0, s>>>(n, v, w);
            SL_TRY(cudaGetLastError());
            SL_TRY(dgetrs_device(trans, n, 1, AF, ldaf, dipiv, v, n, ws, s));
          }
          count_launches(1);
          return cudaGetLastError();
        },
        lw, iw, s, &est));
    iamax_kernel<<<1, 1024, 0, s>>>(x, n, iw + 1, scal + 1);
    count_launches(1);
    double xmax = 0.0;
    SL_TRY(read_sync(&xmax, scal + 1, sizeof(double), s));
    if (xmax != 0.0) ferr[k] = est / xmax;
  }
  return cudaSuccess;
}

cudaError_t dgeequ_device(int m, int n, const double* A, long long lda, double* R, double* C,
                          double* rowcnd, double* colcnd, double* amax, int* info, double* work,
                          int* iw, cudaStream_t s) {
  *info = 0;
  if (m == 0 || n == 0) {
    *rowcnd = 1.0;
    *colcnd = 1.0;
    *amax = 0.0;
    return cudaSuccess;
  }
  const double smlnum = DBL_MIN;  // PDLAMCH 'S'
  const double bignum = 1.0 / smlnum;
  unsigned long long* rbits = reinterpret_cast<unsigned long long*>(work);
  double* scal = work + (m > n ? m : n);
  SL_TRY(cudaMemsetAsync(rbits, 0, sizeof(unsigned long long) * m, s));
  const int rb = (m + 255) / 256;
  int ks = (4 * num_sms() + rb - 1) / rb;
  if (ks < 1) ks = 1;
  if (ks > n) ks = n;
  const int kslice = (n + ks - 1) / ks;
  ks = (n + kslice - 1) / kslice;
  rowmax_abs_kernel<<<dim3(rb, ks), 256, 0, s>>>(m, n, A, lda, kslice, rbits);
  bits_to_double_kernel<<<blocks(m), 256, 0, s>>>(m, rbits, R);
  minmax_kernel<<<1, 1024, 0, s>>>(m, R, bignum, scal, iw);
  count_launches(3);
  SL_TRY(cudaGetLastError());
  double mm[2];
  int z = 0;
  SL_TRY(cudaMemcpyAsync(mm, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  SL_TRY(read_sync(&z, iw, sizeof(int), s));
  *amax = mm[0];
  if (mm[1] == 0.0) {  // first zero row (SRC/pdgeequ.f, loop 50)
    *info = z;
    return cudaSuccess;
  }
  recip_clamp_kernel<<<blocks(m), 256, 0, s>>>(m, R, smlnum, bignum);
  *rowcnd = fmax(mm[1], smlnum) / fmin(mm[0], bignum);
  colmax_scaled_kernel<<<n, 256, 0, s>>>(m, A, lda, R, C);
  minmax_kernel<<<1, 1024, 0, s>>>(n, C, bignum, scal, iw);
  count_launches(3);
  SL_TRY(cudaGetLastError());
  SL_TRY(cudaMemcpyAsync(mm, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
  SL_TRY(read_sync(&z, iw, sizeof(int), s));
  if (mm[1] == 0.0) {  // first zero column: INFO = M + j (loop 110)
    *info = m + z;
    return cudaSuccess;
  }
  recip_clamp_kernel<<<blocks(n), 256, 0, s>>>(n, C, smlnum, bignum);
  count_launches(1);
  *colcnd = fmax(mm[1], smlnum) / fmin(mm[0], bignum);
  return cudaGetLastError();
}

char dlaqge_equed(double rowcnd, double colcnd, double amax) {
  // SMALL = safe minimum / precision (2^-1022 / 2^-52), LARGE = 1 / SMALL, THRESH = 0.1
  const double small = DBL_MIN / DBL_EPSILON;
  const double large = 1.0 / small;
  const double thresh = 0.1;
  if (rowcnd >= thresh && amax >= small && amax <= large) return colcnd >= thresh ? 'N' : 'C';
  return colcnd >= thresh ? 'R' : 'B';
}

cudaError_t dlaqge_device(int m, int n, double* A, long long lda, const double* R, const double* C,
                          char equed, cudaStream_t s) {
  if (m <= 0 || n <= 0 || equed == 'N') return cudaSuccess;
  laqge_kernel<<<blocks((long long)m * n), 256, 0, s>>>(m, n, A, lda, R, C, (int)equed);
  count_launches(1);
  return cudaGetLastError();
}

cudaError_t scale_rows_device(int n, int ncols, double* X, long long ldx, const double* v,
                              cudaStream_t s) {
  if (n <= 0 || ncols <= 0) return cudaSuccess;
  scale_rows_kernel<<<blocks((long long)n * ncols), 256, 0, s>>>(n, ncols, X, ldx, v);
  count_launches(1);
  return cudaGetLastError();
}

}  // namespace sl
