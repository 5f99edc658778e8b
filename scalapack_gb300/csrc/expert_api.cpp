// Host layer of the expert drivers around the LU on a 1x1 grid:
//
//   pdgeequ_  PDGEEQU  (SRC/pdgeequ.f)   row/column scale factors
//   pdlaqge_  PDLAQGE  (SRC/pdlaqge.f)   equilibrates sub(A) when worthwhile
//   pdgerfs_  PDGERFS  (SRC/pdgerfs.f)   refinement, FERR and BERR
//   pdgesvx_  PDGESVX  (SRC/pdgesvx.f)   equilibrate, factor, RCOND, solve,
//                                         refine, unscale
//
// plus device-pointer forms (sl1x1_dgeequ_dev, sl1x1_dgerfs_dev). Argument
// checks follow the reference's order and INFO encoding on a 1x1 grid (every
// INDXG2P / process-row comparison is then equal and drops out); the
// arithmetic runs on the GPU (refine.cu, aux.cu, lu_f64.cu). Host arrays are
// staged into library-owned device buffers as for PDGESV.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/sl1x1.h"
#include "host_state.h"
#include "sl_internal.h"

using namespace sl::host;

namespace {

char upc(char c) { return (c >= 'a' && c <= 'z') ? (char)(c - 32) : c; }

// sub-block (i0, j0 1-based, m x n) of a host array with leading dimension lld
cudaError_t h2d(double* dst, long long ldd, const double* A, int i0, int j0, long long lld, int m,
                int n, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  return cudaMemcpy2DAsync(dst, ldd * sizeof(double), A + (i0 - 1) + (long long)(j0 - 1) * lld,
                           lld * sizeof(double), (size_t)m * sizeof(double), n,
                           cudaMemcpyHostToDevice, s);
}
cudaError_t d2h(double* A, int i0, int j0, long long lld, const double* src, long long ldd, int m,
                int n, cudaStream_t s) {
  if (m <= 0 || n <= 0) return cudaSuccess;
  return cudaMemcpy2DAsync(A + (i0 - 1) + (long long)(j0 - 1) * lld, lld * sizeof(double), src,
                           ldd * sizeof(double), (size_t)m * sizeof(double), n,
                           cudaMemcpyDeviceToHost, s);
}

// IPIV(i0 .. i0+n-1) (global 1-based rows) -> device rows relative to i0
cudaError_t ipiv_to_dev(int* dipiv, const int* IPIV, int i0, int n, cudaStream_t s) {
  std::vector<int> hp((size_t)(n > 0 ? n : 1));
  for (int k = 0; k < n; ++k) hp[k] = IPIV[i0 - 1 + k] - i0;
  cudaError_t e = cudaMemcpyAsync(dipiv, hp.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // hp goes out of scope
  return e;
}
cudaError_t ipiv_to_host(int* IPIV, const int* dipiv, int i0, int n, cudaStream_t s) {
  std::vector<int> hp((size_t)(n > 0 ? n : 1));
  cudaError_t e = cudaMemcpyAsync(hp.data(), dipiv, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  for (int k = 0; k < n; ++k) IPIV[i0 - 1 + k] = i0 + hp[k];
  return cudaSuccess;
}

// The device buffers of one expert call: A (dA2), AF (dA), B (dB), X (dX),
// pivots (dipiv), refinement workspace (drw) and small int scratch.
struct Staging {
  long long ldd = 1;
  int* iw = nullptr;  // 8 ints
  double* rc = nullptr;
};
cudaError_t stage_buffers(int n, int nrhs, Staging* st) {
  st->ldd = round_ld(n);
  const size_t nn = (size_t)st->ldd * (size_t)(n > 0 ? n : 1);
  const size_t nb = (size_t)st->ldd * (size_t)(nrhs > 0 ? nrhs : 1);
  cudaError_t e = grow(&g_dev.dA2, &g_dev.capA2, nn);
  if (e == cudaSuccess) e = grow(&g_dev.dA, &g_dev.capA, nn);
  if (e == cudaSuccess) e = grow(&g_dev.dB, &g_dev.capB, nb);
  if (e == cudaSuccess) e = grow(&g_dev.dX, &g_dev.capX, nb);
  if (e == cudaSuccess) e = grow(&g_dev.dipiv, &g_dev.capP, (size_t)(n > 0 ? n : 1));
  if (e == cudaSuccess) e = grow(&g_dev.dipiv2, &g_dev.capP2, (size_t)n + 16);
  if (e == cudaSuccess) e = grow(&g_dev.drw, &g_dev.capRw, sl::refine_work_doubles(n));
  // R, C, the vector scale of B / X, and the equilibration work (max(m,n) + 4)
  if (e == cudaSuccess) e = grow(&g_dev.drc, &g_dev.capRc, 4 * (size_t)(n > 0 ? n : 1) + 8);
  if (e == cudaSuccess) e = ensure_solve_ws(n, nrhs > 0 ? nrhs : 1);
  st->iw = g_dev.dipiv2 + (n > 0 ? n : 0);
  st->rc = g_dev.drc;
  return e;
}

// PDGERFS argument checks (SRC/pdgerfs.f:334-440) on a 1x1 grid.
int check_gerfs(char trans, int n, int nrhs, int ia, int ja, const int* desca, int iaf, int jaf,
                const int* descaf, int ib, int jb, const int* descb, int ix, int jx,
                const int* descx, int lwork, int liwork, int* lwmin, int* liwmin, bool* lquery) {
  int nprow, npcol, myrow, mycol;
  gridinfo(desca[CTXT_], &nprow, &npcol, &myrow, &mycol);
  int info = 0;
  *lquery = false;
  if (nprow == -1) return -(700 + FCTXT);
  chk1mat(n, 2, n, 2, ia, ja, desca, 7, &info);
  chk1mat(n, 2, n, 2, iaf, jaf, descaf, 11, &info);
  chk1mat(n, 2, nrhs, 3, ib, jb, descb, 16, &info);
  chk1mat(n, 2, nrhs, 3, ix, jx, descx, 20, &info);
  if (info != 0) return info;
  const int iroffa = (ia - 1) % desca[MB_], icoffa = (ja - 1) % desca[NB_];
  const int iroffaf = (iaf - 1) % descaf[MB_], icoffaf = (jaf - 1) % descaf[NB_];
  const int iroffb = (ib - 1) % descb[MB_], icoffb = (jb - 1) % descb[NB_];
  const int iroffx = (ix - 1) % descx[MB_], icoffx = (jx - 1) % descx[NB_];
  const int npmod = numroc(n + iroffa, desca[MB_], 0, 0, 1);
  *lwmin = 3 * npmod;
  *liwmin = npmod;
  *lquery = (lwork == -1 || liwork == -1);
  if (trans != 'N' && trans != 'T' && trans != 'C') info = -1;
  else if (n < 0) info = -2;
  else if (nrhs < 0) info = -3;
  else if (iroffa != 0) info = -5;
  else if (icoffa != 0) info = -6;
  else if (desca[MB_] != desca[NB_]) info = -(700 + FNB);
  else if (desca[MB_] != descaf[MB_]) info = -(1100 + FMB);
  else if (iroffaf != 0) info = -9;
  else if (desca[NB_] != descaf[NB_]) info = -(1100 + FNB);
  else if (icoffaf != 0) info = -10;
  else if (desca[CTXT_] != descaf[CTXT_]) info = -(1100 + FCTXT);
  else if (iroffa != iroffb) info = -14;
  else if (desca[MB_] != descb[MB_]) info = -(1600 + FMB);
  else if (desca[CTXT_] != descb[CTXT_]) info = -(1600 + FCTXT);
  else if (descb[MB_] != descx[MB_]) info = -(2000 + FMB);
  else if (iroffx != 0) info = -18;
  else if (descb[NB_] != descx[NB_]) info = -(2000 + FNB);
  else if (icoffb != icoffx) info = -19;
  else if (desca[CTXT_] != descx[CTXT_]) info = -(2000 + FCTXT);
  else if (lwork < *lwmin && !*lquery) info = -24;
  else if (liwork < *liwmin && !*lquery) info = -26;
  return info;
}

// Device part of PDGERFS once A (dA2), AF (dA), pivots, B (dB) and X (dX)
// are staged; ferr/berr point at FERR(JB) / BERR(JB).
int gerfs_staged(char trans, int n, int nrhs, const Staging& st, double* ferr, double* berr,
                 cudaStream_t s) {
  sl::LuWork w = make_work();
  cudaError_t e = sl::dgerfs_device(trans, n, nrhs, g_dev.dA2, st.ldd, g_dev.dA, st.ldd,
                                    g_dev.dipiv, g_dev.dB, st.ldd, g_dev.dX, st.ldd, ferr, berr, w,
                                    g_dev.drw, st.iw, s);
  return e == cudaSuccess ? 0 : cuda_info(e);
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------- PDGERFS
void pdgerfs_(const char* TRANS, const int* N, const int* NRHS, const double* A, const int* IA,
              const int* JA, const int* DESCA, const double* AF, const int* IAF, const int* JAF,
              const int* DESCAF, const int* IPIV, const double* B, const int* IB, const int* JB,
              const int* DESCB, double* X, const int* IX, const int* JX, const int* DESCX,
              double* FERR, double* BERR, double* WORK, const int* LWORK, int* IWORK,
              const int* LIWORK, int* INFO, size_t TRANS_len) {
  (void)TRANS_len;
  std::lock_guard<std::mutex> lk(g_mu);
  const char trans = upc(TRANS[0]);
  const int n = *N, nrhs = *NRHS;
  int lwmin = 0, liwmin = 0;
  bool lquery = false;
  int info = check_gerfs(trans, n, nrhs, *IA, *JA, DESCA, *IAF, *JAF, DESCAF, *IB, *JB, DESCB, *IX,
                         *JX, DESCX, *LWORK, *LIWORK, &lwmin, &liwmin, &lquery);
  if (info == 0 || lquery) {
    if (lwmin > 0 || lquery) { WORK[0] = (double)lwmin; IWORK[0] = liwmin; }
  }
  if (info != 0) {
    pxerbla(DESCA[CTXT_], "PDGERFS", -info);
    *INFO = info;
    return;
  }
  *INFO = 0;
  if (lquery) return;
  double* ferr = FERR + (*JB - 1);
  double* berr = BERR + (*JB - 1);
  if (n <= 1 || nrhs == 0) {  // SRC/pdgerfs.f:455-461
    for (int k = 0; k < nrhs; ++k) { ferr[k] = 0.0; berr[k] = 0.0; }
    return;
  }
  if (!ensure_device()) { *INFO = cuda_info(cudaErrorNoDevice); return; }
  cudaStream_t s = g_dev.stream;
  Staging st;
  cudaError_t e = stage_buffers(n, nrhs, &st);
  if (e == cudaSuccess) e = h2d(g_dev.dA2, st.ldd, A, *IA, *JA, DESCA[LLD_], n, n, s);
  if (e == cudaSuccess) e = h2d(g_dev.dA, st.ldd, AF, *IAF, *JAF, DESCAF[LLD_], n, n, s);
  if (e == cudaSuccess) e = h2d(g_dev.dB, st.ldd, B, *IB, *JB, DESCB[LLD_], n, nrhs, s);
  if (e == cudaSuccess) e = h2d(g_dev.dX, st.ldd, X, *IX, *JX, DESCX[LLD_], n, nrhs, s);
  if (e == cudaSuccess) e = ipiv_to_dev(g_dev.dipiv, IPIV, *IAF, n, s);
  if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  int r = gerfs_staged(trans, n, nrhs, st, ferr, berr, s);
  if (r != 0) { *INFO = r; return; }
  e = d2h(X, *IX, *JX, DESCX[LLD_], g_dev.dX, st.ldd, n, nrhs, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  WORK[0] = (double)lwmin;
  IWORK[0] = liwmin;
}

// ---------------------------------------------------------------- PDGEEQU
void pdgeequ_(const int* M, const int* N, const double* A, const int* IA, const int* JA,
              const int* DESCA, double* R, double* C, double* ROWCND, double* COLCND, double* AMAX,
              int* INFO) {
  std::lock_guard<std::mutex> lk(g_mu);
  const int m = *M, n = *N;
  int nprow, npcol, myrow, mycol;
  gridinfo(DESCA[CTXT_], &nprow, &npcol, &myrow, &mycol);
  int info = 0;
  if (nprow == -1) info = -(600 + FCTXT);
  else chk1mat(m, 1, n, 2, *IA, *JA, DESCA, 6, &info);
  if (info != 0) {
    pxerbla(DESCA[CTXT_], "PDGEEQU", -info);
    *INFO = info;
    return;
  }
  *INFO = 0;
  if (m == 0 || n == 0) {
    *ROWCND = 1.0;
    *COLCND = 1.0;
    *AMAX = 0.0;
    return;
  }
  if (!ensure_device()) { *INFO = cuda_info(cudaErrorNoDevice); return; }
  cudaStream_t s = g_dev.stream;
  const long long ldd = round_ld(m);
  const int mx = m > n ? m : n;
  cudaError_t e = grow(&g_dev.dA2, &g_dev.capA2, (size_t)ldd * n);
  if (e == cudaSuccess) e = grow(&g_dev.drc, &g_dev.capRc, (size_t)m + n + mx + 8);
  if (e == cudaSuccess) e = grow(&g_dev.dipiv2, &g_dev.capP2, 16);
  if (e == cudaSuccess) e = h2d(g_dev.dA2, ldd, A, *IA, *JA, DESCA[LLD_], m, n, s);
  if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  double* dR = g_dev.drc;
  double* dC = g_dev.drc + m;
  double rowcnd = *ROWCND, colcnd = *COLCND, amax = 0.0;
  int infeq = 0;
  e = sl::dgeequ_device(m, n, g_dev.dA2, ldd, dR, dC, &rowcnd, &colcnd, &amax, &infeq,
                        g_dev.drc + m + n, g_dev.dipiv2, s);
  if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  // R(IA..) always holds the row pass's values; C(JA..) when the column pass ran.
  e = cudaMemcpyAsync(R + (*IA - 1), dR, sizeof(double) * m, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && (infeq == 0 || infeq > m))
    e = cudaMemcpyAsync(C + (*JA - 1), dC, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  *AMAX = amax;
  if (infeq == 0 || infeq > m) *ROWCND = rowcnd;
  if (infeq == 0) *COLCND = colcnd;
  *INFO = infeq;
}

// ---------------------------------------------------------------- PDLAQGE
void pdlaqge_(const int* M, const int* N, double* A, const int* IA, const int* JA,
              const int* DESCA, const double* R, const double* C, const double* ROWCND,
              const double* COLCND, const double* AMAX, char* EQUED, size_t EQUED_len) {
  (void)EQUED_len;
  std::lock_guard<std::mutex> lk(g_mu);
  const int m = *M, n = *N;
  if (m <= 0 || n <= 0) { EQUED[0] = 'N'; return; }
  const char eq = sl::dlaqge_equed(*ROWCND, *COLCND, *AMAX);
  EQUED[0] = eq;
  if (eq == 'N') return;
  if (!ensure_device()) return;  // no INFO argument: the matrix is left as it was
  cudaStream_t s = g_dev.stream;
  const long long ldd = round_ld(m);
  cudaError_t e = grow(&g_dev.dA2, &g_dev.capA2, (size_t)ldd * n);
  if (e == cudaSuccess) e = grow(&g_dev.drc, &g_dev.capRc, (size_t)m + n + 8);
  if (e == cudaSuccess) e = h2d(g_dev.dA2, ldd, A, *IA, *JA, DESCA[LLD_], m, n, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g_dev.drc, R + (*IA - 1), sizeof(double) * m, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g_dev.drc + m, C + (*JA - 1), sizeof(double) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = sl::dlaqge_device(m, n, g_dev.dA2, ldd, g_dev.drc, g_dev.drc + m, eq, s);
  if (e == cudaSuccess) e = d2h(A, *IA, *JA, DESCA[LLD_], g_dev.dA2, ldd, m, n, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    std::fprintf(stderr, "pdlaqge_: CUDA error %d; sub(A) may be partly scaled\n", (int)e);
}

// ---------------------------------------------------------------- PDGESVX
void pdgesvx_(const char* FACT, const char* TRANS, const int* N, const int* NRHS, double* A,
              const int* IA, const int* JA, const int* DESCA, double* AF, const int* IAF,
              const int* JAF, const int* DESCAF, int* IPIV, char* EQUED, double* R, double* C,
              double* B, const int* IB, const int* JB, const int* DESCB, double* X, const int* IX,
              const int* JX, const int* DESCX, double* RCOND, double* FERR, double* BERR,
              double* WORK, const int* LWORK, int* IWORK, const int* LIWORK, int* INFO,
              size_t FACT_len, size_t TRANS_len, size_t EQUED_len) {
  (void)FACT_len;
  (void)TRANS_len;
  (void)EQUED_len;
  std::lock_guard<std::mutex> lk(g_mu);
  const char fact = upc(FACT[0]), trans = upc(TRANS[0]);
  const int n = *N, nrhs = *NRHS, ia = *IA, ja = *JA, iaf = *IAF, jaf = *JAF;
  const int ib = *IB, jb = *JB, ix = *IX, jx = *JX;
  int nprow, npcol, myrow, mycol;
  gridinfo(DESCA[CTXT_], &nprow, &npcol, &myrow, &mycol);
  int info = 0;
  bool nofact = false, equil = false, notran = false, rowequ = false, colequ = false;
  double rowcnd = 1.0, colcnd = 1.0;
  int lwmin = 0, liwmin = 0;
  bool have_min = false, lquery = false;
  // ---- argument checks, SRC/pdgesvx.f:455-656 on a 1x1 grid ----
  if (nprow == -1) {
    info = -(800 + FCTXT);
  } else {
    chk1mat(n, 3, n, 3, ia, ja, DESCA, 8, &info);
    if (fact == 'F') chk1mat(n, 3, n, 3, iaf, jaf, DESCAF, 12, &info);
    chk1mat(n, 3, nrhs, 4, ib, jb, DESCB, 20, &info);
    chk1mat(n, 3, nrhs, 4, ix, jx, DESCX, 24, &info);
    nofact = (fact == 'N');
    equil = (fact == 'E');
    notran = (trans == 'N');
    if (nofact || equil) {
      EQUED[0] = 'N';
    } else {
      const char eq = upc(EQUED[0]);
      rowequ = (eq == 'R' || eq == 'B');
      colequ = (eq == 'C' || eq == 'B');
    }
    const double smlnum = DBL_MIN, bignum = 1.0 / smlnum;
    if (info == 0) {
      const int iroffa = (ia - 1) % DESCA[MB_], iroffaf = (iaf - 1) % DESCAF[MB_];
      const int icoffa = (ja - 1) % DESCA[NB_];
      const int np = n, nq = n;  // NUMROC(N+IROFF, ...) - IROFF on one process
      const int nb = DESCA[NB_];
      const int nqb = (n + iroffa + nb - 1) / nb;
      int conwrk = 2 * np + 2 * nq;
      {
        const int a = nb * 1, b = nq + nb * 1;  // MAX(1, ICEIL(0, 1)) = 1
        int mx = a > b ? a : b;
        if (mx < 2) mx = 2;
        conwrk += mx;
      }
      int rfswrk = 3 * np;
      if (trans == 'N') rfswrk += np + nq + nqb * nb;
      else if (trans == 'T' || trans == 'C') rfswrk += np + nq;
      lwmin = conwrk > rfswrk ? conwrk : rfswrk;
      liwmin = np;
      have_min = true;
      if (!nofact && !equil && fact != 'F') info = -1;
      else if (!notran && trans != 'T' && trans != 'C') info = -2;
      else if (iroffa != 0) info = -6;
      else if (icoffa != 0 || iroffa != icoffa) info = -7;
      else if (DESCA[MB_] != DESCA[NB_]) info = -(800 + FNB);
      else if (iroffaf != 0) info = -10;
      else if (DESCA[CTXT_] != DESCAF[CTXT_]) info = -(1200 + FCTXT);
      else if (fact == 'F' && !(rowequ || colequ || upc(EQUED[0]) == 'N')) info = -13;
      else {
        if (rowequ) {
          double rcmin = bignum, rcmax = 0.0;
          for (int j = 0; j < np; ++j) {
            rcmin = fmin(rcmin, R[ia - 1 + j]);
            rcmax = fmax(rcmax, R[ia - 1 + j]);
          }
          if (rcmin <= 0.0) info = -14;
          else if (n > 0) rowcnd = fmax(rcmin, smlnum) / fmin(rcmax, bignum);
          else rowcnd = 1.0;
        }
        if (colequ && info == 0) {
          double rcmin = bignum, rcmax = 0.0;
          for (int j = 0; j < nq; ++j) {
            rcmin = fmin(rcmin, C[ja - 1 + j]);
            rcmax = fmax(rcmax, C[ja - 1 + j]);
          }
          if (rcmin <= 0.0) info = -15;
          else if (n > 0) colcnd = fmax(rcmin, smlnum) / fmin(rcmax, bignum);
          else colcnd = 1.0;
        }
      }
    }
    if (have_min) { WORK[0] = (double)lwmin; IWORK[0] = liwmin; }
    lquery = (*LWORK == -1 || *LIWORK == -1);
    if (info == 0) {
      if (DESCB[MB_] != DESCA[NB_]) info = -(2000 + FNB);
      else if (DESCA[CTXT_] != DESCB[CTXT_]) info = -(2000 + FCTXT);
      else if (DESCX[MB_] != DESCA[NB_]) info = -(2400 + FNB);
      else if (DESCA[CTXT_] != DESCX[CTXT_]) info = -(2400 + FCTXT);
      else if (*LWORK < lwmin && !lquery) info = -29;
      else if (*LIWORK < liwmin && !lquery) info = -31;
    }
  }
  if (info != 0) {
    pxerbla(DESCA[CTXT_], "PDGESVX", -info);
    *INFO = info;
    return;
  }
  *INFO = 0;
  if (lquery) return;
  double* ferr = FERR + (jb - 1);  // PDGERFS writes FERR/BERR from JB
  double* berr = BERR + (jb - 1);
  if (n == 0) {  // every step is a quick return: RCOND = 1, FERR = BERR = 0
    *RCOND = 1.0;
    for (int k = 0; k < nrhs; ++k) { ferr[k] = 0.0; berr[k] = 0.0; }
    return;
  }
  if (!ensure_device()) { *INFO = cuda_info(cudaErrorNoDevice); return; }
  cudaStream_t s = g_dev.stream;
  Staging st;
  cudaError_t e = stage_buffers(n, nrhs, &st);
  if (e == cudaSuccess) e = h2d(g_dev.dA2, st.ldd, A, ia, ja, DESCA[LLD_], n, n, s);
  if (e == cudaSuccess) e = h2d(g_dev.dB, st.ldd, B, ib, jb, DESCB[LLD_], n, nrhs, s);
  if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  double* dR = st.rc;
  double* dC = st.rc + n;
  double* dv = st.rc + 2 * (size_t)n;  // a scale vector for B or X
  bool a_scaled = false, b_scaled = false;
  auto fail = [&](cudaError_t err) { *INFO = cuda_info(err); };
  // ---- 1. equilibration (PDGEEQU + PDLAQGE) ----
  if (equil) {
    double rc = 1.0, cc = 1.0, amax = 0.0;
    int infequ = 0;
    e = sl::dgeequ_device(n, n, g_dev.dA2, st.ldd, dR, dC, &rc, &cc, &amax, &infequ,
                          st.rc + 2 * (size_t)n, st.iw, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(R + (ia - 1), dR, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && (infequ == 0 || infequ > n))
      e = cudaMemcpyAsync(C + (ja - 1), dC, sizeof(double) * n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(e);
    if (infequ == 0) {
      rowcnd = rc;
      colcnd = cc;
      const char eq = sl::dlaqge_equed(rowcnd, colcnd, amax);
      EQUED[0] = eq;
      e = sl::dlaqge_device(n, n, g_dev.dA2, st.ldd, dR, dC, eq, s);
      if (e != cudaSuccess) return fail(e);
      rowequ = (eq == 'R' || eq == 'B');
      colequ = (eq == 'C' || eq == 'B');
      a_scaled = (eq != 'N');
    }
  }
  // ---- scale the right-hand side: R(IB..) rows, or C(JA..) for op = T ----
  if ((notran && rowequ) || (!notran && colequ)) {
    const double* v = notran ? R + (ib - 1) : C + (ja - 1);
    e = cudaMemcpyAsync(dv, v, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = sl::scale_rows_device(n, nrhs, g_dev.dB, st.ldd, dv, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(e);
    b_scaled = true;
  }
  auto write_back = [&]() -> cudaError_t {
    cudaError_t err = cudaSuccess;
    if (a_scaled) err = d2h(A, ia, ja, DESCA[LLD_], g_dev.dA2, st.ldd, n, n, s);
    if (err == cudaSuccess && b_scaled) err = d2h(B, ib, jb, DESCB[LLD_], g_dev.dB, st.ldd, n, nrhs, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    return err;
  };
  // ---- 2. factor AF = P L U (PDLACPY + PDGETRF), or take the given factors ----
  sl::LuWork w = make_work();
  if (nofact || equil) {
    e = cudaMemcpy2DAsync(g_dev.dA, st.ldd * sizeof(double), g_dev.dA2, st.ldd * sizeof(double),
                          (size_t)n * sizeof(double), n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return fail(e);
    if (DESCAF[M_] == 1 && n == 1) {
      // PDGETRF on a 1x1 global matrix returns at once with IPIV = 1
      const int zero = 0;
      e = cudaMemcpyAsync(g_dev.dipiv, &zero, sizeof(int), cudaMemcpyHostToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e != cudaSuccess) return fail(e);
    } else {
      ensure_oz(n, n, DESCAF[NB_]);
      e = sl::dgetrf_device(n, n, g_dev.dA, st.ldd, g_dev.dipiv, DESCAF[NB_], w, s);
      if (e == cudaErrorInvalidValue) { *INFO = -30000; return; }
      if (e != cudaSuccess) return fail(e);
      int finfo = 0;
      read_factor_info(s, n, &finfo);
      if (finfo <= -10000) { *INFO = finfo; return; }
      info = finfo;
    }
    e = d2h(AF, iaf, jaf, DESCAF[LLD_], g_dev.dA, st.ldd, n, n, s);
    if (e == cudaSuccess) e = ipiv_to_host(IPIV, g_dev.dipiv, iaf, n, s);
    if (e != cudaSuccess) return fail(e);
    if (info != 0) {  // singular: RCOND = 0, no solution (SRC/pdgesvx.f:737-742)
      if (info > 0) *RCOND = 0.0;
      e = write_back();
      *INFO = (e == cudaSuccess) ? info : cuda_info(e);
      return;
    }
  } else {
    e = h2d(g_dev.dA, st.ldd, AF, iaf, jaf, DESCAF[LLD_], n, n, s);
    if (e == cudaSuccess) e = ipiv_to_dev(g_dev.dipiv, IPIV, iaf, n, s);
    if (e != cudaSuccess) return fail(e);
  }
  // ---- 3. RCOND from PDLANGE + PDGECON ----
  {
    const char norm = notran ? '1' : 'I';
    e = grow(&g_dev.daux, &g_dev.capAux, 3 * (size_t)n + 16);
    double anorm = 0.0;
    if (e == cudaSuccess) e = sl::dlange_device(norm, n, n, g_dev.dA2, st.ldd, g_dev.daux, g_dev.daux + n + 4, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(&anorm, g_dev.daux + n + 4, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    double rcond = 0.0;
    if (e == cudaSuccess)
      e = sl::dgecon_device(notran, n, g_dev.dA, st.ldd, anorm, &rcond, g_dev.daux,
                            reinterpret_cast<int*>(g_dev.daux + 3 * (size_t)n + 8), s);
    if (e != cudaSuccess) return fail(e);
    *RCOND = rcond;
    if (rcond < DBL_EPSILON * 0.5) {  // singular to working precision (INFO = IA + N)
      e = write_back();
      *INFO = (e == cudaSuccess) ? ia + n : cuda_info(e);
      return;
    }
  }
  // ---- 4. X = B, PDGETRS ----
  e = cudaMemcpy2DAsync(g_dev.dX, st.ldd * sizeof(double), g_dev.dB, st.ldd * sizeof(double),
                        (size_t)n * sizeof(double), nrhs, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = sl::dgetrs_device(trans, n, nrhs, g_dev.dA, st.ldd, g_dev.dipiv, g_dev.dX, st.ldd, w, s);
  if (e != cudaSuccess) return fail(e);
  // ---- 5. PDGERFS (N <= 1 returns FERR = BERR = 0 without refining) ----
  if (n <= 1 || nrhs == 0) {
    for (int k = 0; k < nrhs; ++k) { ferr[k] = 0.0; berr[k] = 0.0; }
  } else {
    const int r = gerfs_staged(trans, n, nrhs, st, ferr, berr, s);
    if (r != 0) { *INFO = r; return; }
  }
  // ---- 6. back to the original system: X = diag(C) X (op = N) or diag(R) X ----
  // (R from IX as the reference indexes it; C from JA; FERR from JX)
  if ((notran && colequ) || (!notran && rowequ)) {
    const double* v = notran ? C + (ja - 1) : R + (ix - 1);
    e = cudaMemcpyAsync(dv, v, sizeof(double) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = sl::scale_rows_device(n, nrhs, g_dev.dX, st.ldd, dv, s);
    if (e != cudaSuccess) return fail(e);
    const double cnd = notran ? colcnd : rowcnd;
    for (int k = 0; k < nrhs; ++k) FERR[jx - 1 + k] = FERR[jx - 1 + k] / cnd;
  }
  e = d2h(X, ix, jx, DESCX[LLD_], g_dev.dX, st.ldd, n, nrhs, s);
  if (e == cudaSuccess) e = write_back();
  if (e != cudaSuccess) return fail(e);
  WORK[0] = (double)lwmin;
  IWORK[0] = liwmin;
  *INFO = 0;
}

// ---------------------------------------------------------------- device forms
int sl1x1_dgeequ_dev(int m, int n, const double* dA, long long ldda, double* dR, double* dC,
                     double* rowcnd, double* colcnd, double* amax, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (ldda < (m > 1 ? m : 1)) return -4;
  if (m == 0 || n == 0) { *rowcnd = 1.0; *colcnd = 1.0; *amax = 0.0; return 0; }
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  cudaStream_t s = (cudaStream_t)stream;
  const int mx = m > n ? m : n;
  cudaError_t e = grow(&g_dev.drc, &g_dev.capRc, (size_t)mx + 8);
  if (e == cudaSuccess) e = grow(&g_dev.dipiv2, &g_dev.capP2, 16);
  if (e != cudaSuccess) return cuda_info(e);
  int info = 0;
  e = sl::dgeequ_device(m, n, dA, ldda, dR, dC, rowcnd, colcnd, amax, &info, g_dev.drc,
                        g_dev.dipiv2, s);
  return e == cudaSuccess ? info : cuda_info(e);
}

int sl1x1_dgerfs_dev(char trans, int n, int nrhs, const double* dA, long long ldda,
                     const double* dAF, long long lddaf, const int* dipiv, const double* dB,
                     long long lddb, double* dX, long long lddx, double* ferr, double* berr,
                     void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  const char t = upc(trans);
  if (t != 'N' && t != 'T' && t != 'C') return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (ldda < (n > 1 ? n : 1)) return -5;
  if (lddaf < (n > 1 ? n : 1)) return -7;
  if (lddb < (n > 1 ? n : 1)) return -10;
  if (lddx < (n > 1 ? n : 1)) return -12;
  if (n <= 1 || nrhs == 0) {
    for (int k = 0; k < nrhs; ++k) { ferr[k] = 0.0; berr[k] = 0.0; }
    return 0;
  }
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = grow(&g_dev.dipiv2, &g_dev.capP2, (size_t)n + 16);
  if (e == cudaSuccess) e = grow(&g_dev.drw, &g_dev.capRw, sl::refine_work_doubles(n));
  if (e == cudaSuccess) e = ensure_solve_ws(n, 1);
  if (e == cudaSuccess) e = sl::ipiv_shift(dipiv, g_dev.dipiv2, n, -1, s);  // LAPACK 1-based -> 0-based
  if (e != cudaSuccess) return cuda_info(e);
  sl::LuWork w = make_work();
  e = sl::dgerfs_device(t, n, nrhs, dA, ldda, dAF, lddaf, g_dev.dipiv2, dB, lddb, dX, lddx, ferr,
                        berr, w, g_dev.drw, g_dev.dipiv2 + n, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? 0 : cuda_info(e);
}

}  // extern "C"
