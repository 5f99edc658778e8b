// Routines around the LU factors (the next rows of the LU path):
//   PDLANGE  (SRC/pdlange.f)  matrix norms 'M', '1'/'O', 'I', 'F'/'E'
//   PDGECON  (SRC/pdgecon.f)  reciprocal condition number estimate from the LU
//            factors, 1-norm or infinity-norm, with the Hager / Higham
//            estimator that PDLACON implements (Higham, "FORTRAN codes for
//            estimating the one-norm of a real or complex matrix", ACM TOMS
//            14(4), 1988, Algorithm 4.1): products with inv(U) inv(L) and its
//            transpose are triangular solves on the GPU; the estimator's
//            control flow runs on the host and reads back scalars only.
//   PDGETRI  (SRC/pdgetri.f)  inverse from the LU factors: INFO = first
//            exactly-zero U(i,i) (PDTRTRI's test), else inv(A) = solve(A, I)
//            with the FP64 solve kernels (the same matrix the reference's
//            inv(U)-then-inv(A)*L sequence produces).
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "common.cuh"
#include "lu_kernels.cuh"
#include "sl_internal.h"

namespace sl {

// ---------------------------------------------------------------- norms
__device__ __forceinline__ double nan_max(double a, double b) {
  return (a != a || b > a) ? (b != b ? b : (a != a ? a : b)) : a;
}

// out[c] = sum_i |A(i,c)|, one CTA per column.
__global__ void colsum_abs_kernel(const double* __restrict__ A, long long lda, int m, double* out) {
  __shared__ double sm[32];
  const int c = blockIdx.x;
  double s = 0.0;
  for (int i = threadIdx.x; i < m; i += blockDim.x) s += fabs(A[i + (long long)c * lda]);
  for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (threadIdx.x == 0) out[c] = s;
  }
}

// out[i] = sum_j |A(i,j)| (kind 0) or max_j |A(i,j)| (kind 1), one thread per row.
__global__ void rowred_abs_kernel(const double* __restrict__ A, long long lda, int m, int n,
                                  int kind, double* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  double s = 0.0;
  for (int j = 0; j < n; ++j) {
    const double v = fabs(A[i + (long long)j * lda]);
    s = kind == 0 ? s + v : nan_max(s, v);
  }
  out[i] = s;
}

// out[i] = sum_j (A(i,j)/scale)^2 with scale read from device memory.
__global__ void rowsumsq_kernel(const double* __restrict__ A, long long lda, int m, int n,
                                const double* scale, double* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const double sc = scale[0];
  double s = 0.0;
  if (sc > 0.0 && isfinite(sc))
    for (int j = 0; j < n; ++j) {
      const double v = A[i + (long long)j * lda] / sc;
      s = fma(v, v, s);
    }
  out[i] = s;
}

// One-CTA reductions of a length-k vector: max (NaN propagates) or sum.
__global__ void vec_reduce_kernel(const double* __restrict__ v, int k, int kind, double* out) {
  __shared__ double sm[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < k; i += blockDim.x) s = kind == 0 ? nan_max(s, v[i]) : s + v[i];
  for (int off = 16; off > 0; off >>= 1) {
    const double o = __shfl_xor_sync(0xffffffffu, s, off);
    s = kind == 0 ? nan_max(s, o) : s + o;
  }
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) {
      const double o = __shfl_xor_sync(0xffffffffu, s, off);
      s = kind == 0 ? nan_max(s, o) : s + o;
    }
    if (threadIdx.x == 0) out[0] = s;
  }
}

cudaError_t dlange_device(char norm, int m, int n, const double* A, long long lda, double* work,
                          double* result, cudaStream_t s) {
  // work: max(m, n) + 2 doubles
  if (m <= 0 || n <= 0) {
    const double z = 0.0;
    return cudaMemcpyAsync(result, &z, sizeof(double), cudaMemcpyHostToDevice, s);
  }
  const char u = (norm >= 'a' && norm <= 'z') ? (char)(norm - 32) : norm;
  if (u == 'M') {
    rowred_abs_kernel<<<(m + 255) / 256, 256, 0, s>>>(A, lda, m, n, 1, work);
    vec_reduce_kernel<<<1, 1024, 0, s>>>(work, m, 0, result);
    count_launches(2);
  } else if (u == 'O' || u == '1') {
    colsum_abs_kernel<<<n, 256, 0, s>>>(A, lda, m, work);
    vec_reduce_kernel<<<1, 1024, 0, s>>>(work, n, 0, result);
    count_launches(2);
  } else if (u == 'I') {
    rowred_abs_kernel<<<(m + 255) / 256, 256, 0, s>>>(A, lda, m, n, 0, work);
    vec_reduce_kernel<<<1, 1024, 0, s>>>(work, m, 0, result);
    count_launches(2);
  } else {  // 'F' / 'E': scale * sqrt(sum((a/scale)^2)), scale = max |a|
    double* scale = work + (m > n ? m : n);
    rowred_abs_kernel<<<(m + 255) / 256, 256, 0, s>>>(A, lda, m, n, 1, work);
    vec_reduce_kernel<<<1, 1024, 0, s>>>(work, m, 0, scale);
    rowsumsq_kernel<<<(m + 255) / 256, 256, 0, s>>>(A, lda, m, n, scale, work);
    vec_reduce_kernel<<<1, 1024, 0, s>>>(work, m, 1, scale + 1);
    count_launches(4);
    double h[2];
    SL_TRY(cudaMemcpyAsync(h, scale, 2 * sizeof(double), cudaMemcpyDeviceToHost, s));
    SL_TRY(cudaStreamSynchronize(s));
    const double v = (h[0] > 0.0 && std::isfinite(h[0])) ? h[0] * std::sqrt(h[1]) : h[0];
    return cudaMemcpyAsync(result, &v, sizeof(double), cudaMemcpyHostToDevice, s);
  }
  return cudaGetLastError();
}

// ------------------------------------------------------- condition estimate
// y(i) = sign(x(i)) as +-1 (0 counts as +); *changed = 1 if any sign differs
// from the previous sign vector `prev`; asum[0] = sum |x|.
__global__ void sign_kernel(const double* __restrict__ x, int n, double* xi,
                            const double* __restrict__ prev, int use_prev, int* changed) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double sgn = x[i] >= 0.0 ? 1.0 : -1.0;
  if (use_prev && prev[i] != sgn) *changed = 1;
  xi[i] = sgn;
}

// x = e_j
__global__ void unit_vec_kernel(double* x, int n, const int* j) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = (i == *j) ? 1.0 : 0.0;
}

// x(i) = (-1)^i (1 + i/(n-1))
__global__ void altsgn_kernel(double* x, int n) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = ((i & 1) ? -1.0 : 1.0) * (1.0 + (double)i / (double)(n - 1));
}

__global__ void fill_kernel(double* x, int n, double v) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

// First index of the largest |z(i)| (IDAMAX), one CTA.
__global__ void iamax_kernel(const double* __restrict__ z, int n, int* jout, double* vout) {
  __shared__ double sk[32];
  __shared__ int sr[32];
  double key = -2.0;
  int row = 0x7fffffff;
  for (int i = threadIdx.x; i < n; i += blockDim.x) amax_combine(key, row, amax_key(z[i]), i);
  warp_amax(key, row);
  if ((threadIdx.x & 31) == 0) { sk[threadIdx.x >> 5] = key; sr[threadIdx.x >> 5] = row; }
  __syncthreads();
  if (threadIdx.x < 32) {
    key = threadIdx.x < (blockDim.x >> 5) ? sk[threadIdx.x] : -2.0;
    row = threadIdx.x < (blockDim.x >> 5) ? sr[threadIdx.x] : 0x7fffffff;
    warp_amax(key, row);
    if (threadIdx.x == 0) {
      if (row == 0x7fffffff) row = 0;
      *jout = row;
      *vout = fabs(z[row]);
    }
  }
}

// y = op x with op = inv(U) inv(L) (trans 0) or its transpose (trans 1), in place.
static cudaError_t apply_inv(bool trans, int n, const double* LU, long long lda, double* x,
                             cudaStream_t s) {
  if (!trans) {
    SL_TRY(tri_solve<double>(true, false, true, n, 1, LU, lda, x, n, s));
    return tri_solve<double>(false, false, false, n, 1, LU, lda, x, n, s);
  }
  SL_TRY(tri_solve<double>(false, true, false, n, 1, LU, lda, x, n, s));
  return tri_solve<double>(true, true, true, n, 1, LU, lda, x, n, s);
}

// Estimate ||B||_1 with B = inv(U)inv(L) (onenrm) or its transpose (infinity
// norm of inv(A)). work: 3*n + 8 doubles; iw: 4 ints.
// Hager's estimate of the 1-norm of an n x n operator B given only products
// (the reverse-communication loop of PDLACON, SRC/pdlacon.f, restated as a
// host-driven loop): apply(true, x) overwrites x with B x, apply(false, x)
// with B^T x. work holds 3n + 4 doubles, iw 2 ints; n >= 2.
cudaError_t lacon_estimate(int n, const LaconApply& apply, double* work, int* iw, cudaStream_t s,
                           double* est_out) {
  double* x = work;
  double* xi = work + n;
  double* tmp = work + 2 * (size_t)n;
  double* scal = work + 3 * (size_t)n;  // [0] sum |y|, [1] |z_j|
  const unsigned g = (unsigned)((n + 255) / 256);
  auto asum = [&](const double* v, double* out) -> cudaError_t {
    rowred_abs_kernel<<<g, 256, 0, s>>>(v, n, n, 1, 0, tmp);  // |v_i| (one column)
    vec_reduce_kernel<<<1, 1024, 0, s>>>(tmp, n, 1, out);
    count_launches(2);
    return cudaGetLastError();
  };
  auto read = [&](void* dst, const void* src, size_t b) -> cudaError_t {
    SL_TRY(cudaMemcpyAsync(dst, src, b, cudaMemcpyDeviceToHost, s));
    return cudaStreamSynchronize(s);
  };
  // x = (1/n, ..., 1/n); y = B x
  fill_kernel<<<g, 256, 0, s>>>(x, n, 1.0 / n);
  count_launches(1);
  SL_TRY(apply(true, x));
  SL_TRY(asum(x, scal));
  double est = 0.0;
  SL_TRY(read(&est, scal, sizeof(double)));
  // xi = sign(y); z = B^T xi
  SL_TRY(cudaMemsetAsync(iw, 0, sizeof(int), s));
  sign_kernel<<<g, 256, 0, s>>>(x, n, xi, xi, 0, iw);
  SL_TRY(cudaMemcpyAsync(x, xi, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  count_launches(1);
  SL_TRY(apply(false, x));
  iamax_kernel<<<1, 1024, 0, s>>>(x, n, iw + 1, scal + 1);
  count_launches(1);
  int iter = 2;
  for (;;) {
    int j = 0;
    SL_TRY(read(&j, iw + 1, sizeof(int)));
    // x = e_j; y = B x
    unit_vec_kernel<<<g, 256, 0, s>>>(x, n, iw + 1);
    count_launches(1);
    SL_TRY(apply(true, x));
    const double est_old = est;
    SL_TRY(asum(x, scal));
    SL_TRY(read(&est, scal, sizeof(double)));
    SL_TRY(cudaMemsetAsync(iw, 0, sizeof(int), s));
    sign_kernel<<<g, 256, 0, s>>>(x, n, tmp + 0, xi, 1, iw);  // signs into tmp, compare with xi
    count_launches(1);
    int changed = 0;
    SL_TRY(read(&changed, iw, sizeof(int)));
    if (!changed || est <= est_old) break;  // repeated sign vector or no growth
    SL_TRY(cudaMemcpyAsync(xi, tmp, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    SL_TRY(cudaMemcpyAsync(x, xi, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    SL_TRY(apply(false, x));
    double zlast = 0.0;
    // |z(jlast)| of the new z, then the new argmax
    SL_TRY(cudaMemcpyAsync(&zlast, x + j, sizeof(double), cudaMemcpyDeviceToHost, s));
    iamax_kernel<<<1, 1024, 0, s>>>(x, n, iw + 1, scal + 1);
    count_launches(1);
    double zj = 0.0;
    SL_TRY(read(&zj, scal + 1, sizeof(double)));
    // continue while the new maximal |z_j| differs from z at the previous j
    // (the signed value, as the estimator compares it) and fewer than 5 steps
    if (zlast == zj || iter >= 5) break;
    ++iter;
  }
  // alternative estimate
  altsgn_kernel<<<g, 256, 0, s>>>(x, n);
  count_launches(1);
  SL_TRY(apply(true, x));
  SL_TRY(asum(x, scal));
  double alt = 0.0;
  SL_TRY(read(&alt, scal, sizeof(double)));
  alt = 2.0 * alt / (3.0 * n);
  if (alt > est) est = alt;
  *est_out = est;
  return cudaSuccess;
}

cudaError_t dgecon_device(bool onenrm, int n, const double* LU, long long lda, double anorm,
                          double* rcond, double* work, int* iw, cudaStream_t s) {
  *rcond = 0.0;
  if (n == 0) { *rcond = 1.0; return cudaSuccess; }
  if (anorm == 0.0) return cudaSuccess;
  if (n == 1) { *rcond = 1.0; return cudaSuccess; }
  const bool t1 = !onenrm;  // KASE 1 applies B, KASE 2 applies B^T
  double est = 0.0;
  SL_TRY(lacon_estimate(
      n, [&](bool kase1, double* x) { return apply_inv(kase1 ? t1 : !t1, n, LU, lda, x, s); }, work,
      iw, s, &est));
  if (est != 0.0 && std::isfinite(est)) *rcond = (1.0 / est) / anorm;
  return cudaSuccess;
}

// ---------------------------------------------------------------- inverse
// first zero on the diagonal of U: *out = min(i+1) with U(i,i) == 0, else n+1
__global__ void diag_zero_kernel(const double* __restrict__ A, long long lda, int n, int* out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && A[i + i * lda] == 0.0) atomicMin(out, (int)i + 1);
}

__global__ void identity_kernel(double* X, long long ldx, int n) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)n * n) return;
  const long long i = idx % n, j = idx / n;
  X[i + j * ldx] = (i == j) ? 1.0 : 0.0;
}

// Inverse of A from its factors (dA holds L\U, dipiv 0-based). X: n x n
// workspace (ld n). Returns INFO through *info (0 or first zero U(i,i)).
cudaError_t dgetri_device(int n, double* dA, long long lda, const int* dipiv, double* X,
                          const LuWork& ws, int* dflag, int* info, cudaStream_t s) {
  *info = 0;
  if (n <= 0) return cudaSuccess;
  const int big = n + 1;
  SL_TRY(cudaMemcpyAsync(dflag, &big, sizeof(int), cudaMemcpyHostToDevice, s));
  diag_zero_kernel<<<(n + 255) / 256, 256, 0, s>>>(dA, lda, n, dflag);
  count_launches(1);
  int first = big;
  SL_TRY(cudaMemcpyAsync(&first, dflag, sizeof(int), cudaMemcpyDeviceToHost, s));
  SL_TRY(cudaStreamSynchronize(s));
  if (first <= n) { *info = first; return cudaSuccess; }
  const long long tot = (long long)n * n;
  identity_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(X, n, n);
  count_launches(1);
  SL_TRY(dgetrs_device('N', n, n, dA, lda, dipiv, X, n, ws, s));
  return cudaMemcpy2DAsync(dA, lda * sizeof(double), X, n * sizeof(double), n * sizeof(double), n,
                           cudaMemcpyDeviceToDevice, s);
}

}  // namespace sl
