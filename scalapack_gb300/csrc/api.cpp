// Host layer of libsl1x1gpu.so: the reference-facing C ABI.
//
//  * argument validation with the reference's INFO codes (TOOLS/chk1mat.f,
//    SRC/pdgetrf.f:170-197, SRC/pdgetrs.f:186-236, SRC/pdgesv.f:181-221) and
//    PXERBLA-format messages (PBLAS/SRC/PTZBLAS/pxerbla.f:57-58);
//  * Fortran-ABI PDGETRF / PDGETRS / PDGESV that stage sub(A), sub(B) and IPIV
//    between host memory and library-owned device buffers;
//  * a 1x1 BLACS shim, DESCINIT and NUMROC so that callers link without MPI;
//  * device-pointer entry points for callers whose data already lives in HBM.
// No routine falls back to the CPU: without a usable GPU every call returns an
// INFO <= -10000.
#include <cuda_runtime.h>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/sl1x1.h"
#include "host_state.h"
#include "sl_internal.h"

namespace sl {
namespace host {

std::mutex g_mu;       // device state and the LU entry points
std::mutex g_grid_mu;  // the 1x1 BLACS shim's context table

// ---------------------------------------------------------------- BLACS shim
struct Grid {
  bool live = false;
  int nprow = -1, npcol = -1;
};
std::vector<Grid> g_grids;

void shim_gridinfo(int ictxt, int* nprow, int* npcol, int* myrow, int* mycol) {
  std::lock_guard<std::mutex> lk(g_grid_mu);
  if (ictxt >= 0 && ictxt < (int)g_grids.size() && g_grids[ictxt].live &&
      g_grids[ictxt].nprow == 1 && g_grids[ictxt].npcol == 1) {
    *nprow = 1; *npcol = 1; *myrow = 0; *mycol = 0;
  } else {
    *nprow = -1; *npcol = -1; *myrow = -1; *mycol = -1;
  }
}

// Grid query used by the LU routines. It goes through the exported
// blacs_gridinfo_ symbol, so a real BLACS linked ahead of this library
// answers instead of the shim. Any grid other than 1x1 is reported as an
// invalid context (NPROW = -1): the GPU path computes on one process only.
void gridinfo(int ictxt, int* nprow, int* npcol, int* myrow, int* mycol) {
  int c = ictxt;
  blacs_gridinfo_(&c, nprow, npcol, myrow, mycol);
  if (*nprow != 1 || *npcol != 1) {
    *nprow = -1; *npcol = -1; *myrow = -1; *mycol = -1;
  }
}

int numroc(int n, int nb, int iproc, int isrcproc, int nprocs) {
  // TOOLS/numroc.f:53-76
  int mydist = (nprocs + iproc - isrcproc) % nprocs;
  int nblocks = n / nb;
  int r = (nblocks / nprocs) * nb;
  int extra = nblocks % nprocs;
  if (mydist < extra) r += nb;
  else if (mydist == extra) r += n % nb;
  return r;
}

void pxerbla(int ictxt, const char* name, int info) {
  int nprow, npcol, myrow, mycol;
  gridinfo(ictxt, &nprow, &npcol, &myrow, &mycol);
  // FORMAT( '{', I5, ',', I5, '}:  On entry to ', A, ' parameter number ', I4, ' had an illegal value' )
  std::printf("{%5d,%5d}:  On entry to %s parameter number %4d had an illegal value\n", myrow,
              mycol, name, info);
  std::fflush(stdout);
}

// CHK1MAT (TOOLS/chk1mat.f): checks one distributed-matrix argument and folds
// the result into INFO with the reference's encoding (smallest position wins).
void chk1mat(int ma, int mapos0, int na, int napos0, int ia, int ja, const int* desca,
             int descapos0, int* info) {
  const int DESCMULT = 100, BIGNUM = DESCMULT * DESCMULT;
  if (*info >= 0) *info = BIGNUM;
  else if (*info < -DESCMULT) *info = -*info;
  else *info = -*info * DESCMULT;
  const int mapos = mapos0 * DESCMULT, napos = napos0 * DESCMULT;
  const int iapos = (descapos0 - 2) * DESCMULT, japos = (descapos0 - 1) * DESCMULT;
  const int descapos = descapos0 * DESCMULT;
  int nprow, npcol, myrow, mycol;
  gridinfo(desca[CTXT_], &nprow, &npcol, &myrow, &mycol);
  auto mn = [&](int v) { if (v < *info) *info = v; };
  if (desca[DTYPE_] != 1) mn(descapos + FDTYPE);
  else if (ma < 0) mn(mapos);
  else if (na < 0) mn(napos);
  else if (ia < 1) mn(iapos);
  else if (ja < 1) mn(japos);
  else if (desca[MB_] < 1) mn(descapos + FMB);
  else if (desca[NB_] < 1) mn(descapos + FNB);
  else if (desca[RSRC_] < 0 || desca[RSRC_] >= nprow) mn(descapos + FRSRC);
  else if (desca[CSRC_] < 0 || desca[CSRC_] >= npcol) mn(descapos + FCSRC);
  else if (desca[LLD_] < 1) mn(descapos + FLLD);
  else if (desca[LLD_] < numroc(desca[M_], desca[MB_], myrow, desca[RSRC_], nprow)) {
    if (numroc(desca[N_], desca[NB_], mycol, desca[CSRC_], npcol) > 0) mn(descapos + FLLD);
  }
  if (ma == 0 || na == 0) {
    if (desca[M_] < 0) mn(descapos + FM);
    if (desca[N_] < 0) mn(descapos + FN);
  } else {
    if (desca[M_] < 1) mn(descapos + FM);
    else if (desca[N_] < 1) mn(descapos + FN);
    else {
      if (ia > desca[M_]) mn(iapos);
      else if (ja > desca[N_]) mn(japos);
      else {
        if (ia + ma - 1 > desca[M_]) mn(mapos);
        if (ja + na - 1 > desca[N_]) mn(napos);
      }
    }
  }
  if (*info == BIGNUM) *info = 0;
  else if (*info % DESCMULT == 0) *info = -*info / DESCMULT;
  else *info = -*info;
}

// ------------------------------------------------------------- device state
DevState g_dev;
int g_default_nb = 256;
double g_ir_cost_ratio = 3.5;  // mixed solver: FP64 cost / low-precision factor time
bool g_lookahead = true;
bool g_split_step = true;  // the next panel's columns on the panel's stream
int g_fail_alloc_in = -1;
int g_copy_chunks = 8;  // column chunks of A's host-to-device copy (<= 1: one copy)

int cuda_info(cudaError_t e) { return -10000 - (int)e; }

bool ensure_device() {
  if (g_dev.init) return g_dev.ok;
  g_dev.init = true;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) return false;
  if (cudaGetDevice(&g_dev.device) != cudaSuccess) return false;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, g_dev.device) != cudaSuccess) return false;
  if (prop.major != 10 || prop.minor != 3) {
    std::fprintf(stderr, "sl1x1: device %d is sm_%d%d; this library is built for sm_103a only\n",
                 g_dev.device, prop.major, prop.minor);
    return false;
  }
  if (cudaStreamCreateWithFlags(&g_dev.stream, cudaStreamNonBlocking) != cudaSuccess) return false;
  {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&g_dev.aux, cudaStreamNonBlocking, hi) != cudaSuccess) return false;
    if (cudaEventCreateWithFlags(&g_dev.ev_next, cudaEventDisableTiming) != cudaSuccess) return false;
    if (cudaEventCreateWithFlags(&g_dev.ev_panel, cudaEventDisableTiming) != cudaSuccess) return false;
    if (cudaStreamCreateWithFlags(&g_dev.h2d, cudaStreamNonBlocking) != cudaSuccess) return false;
    if (cudaEventCreateWithFlags(&g_dev.ev_h2d, cudaEventDisableTiming) != cudaSuccess) return false;
    for (cudaEvent_t& ev : g_dev.ev_cols)
      if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return false;
  }
  if (cudaMalloc(&g_dev.dsmall, 16 * sizeof(int)) != cudaSuccess) return false;
  if (cudaMalloc(&g_dev.dcand, sl::panel_cand_doubles() * sizeof(double)) != cudaSuccess) return false;
  if (cudaMalloc(&g_dev.dplan, 2 * sl::kSwapPlanInts * sizeof(int)) != cudaSuccess) return false;
  g_dev.ok = true;
  return true;
}

void release_all() {
  if (!g_dev.ok) return;
  cudaFree(g_dev.dA); cudaFree(g_dev.dB); cudaFree(g_dev.dipiv); cudaFree(g_dev.dsmall);
  cudaFree(g_dev.dcand); cudaFree(g_dev.dplan); cudaFree(g_dev.dperm); cudaFree(g_dev.dbswap);
  cudaFree(g_dev.dA16); cudaFree(g_dev.dB16); cudaFree(g_dev.dcolexp);
  cudaFree(g_dev.dF); cudaFree(g_dev.dpermx); cudaFree(g_dev.dR); cudaFree(g_dev.dD);
  cudaFree(g_dev.dXf); cudaFree(g_dev.dXt); cudaFree(g_dev.dcm); cudaFree(g_dev.dV);
  cudaFree(g_dev.dw); cudaFree(g_dev.dAx); cudaFree(g_dev.dh); cudaFree(g_dev.dAcopy);
  cudaFree(g_dev.dchain); cudaFree(g_dev.dsplitk); cudaFree(g_dev.daux); cudaFree(g_dev.ddinv);
  cudaFree(g_dev.dA2); cudaFree(g_dev.dX); cudaFree(g_dev.drw); cudaFree(g_dev.drc);
  cudaFree(g_dev.dipiv2); cudaFree(g_dev.doz); cudaFree(g_dev.doz2); cudaFree(g_dev.ddinv64);
  cudaFree(g_dev.ddinvs);
  cudaFree(g_dev.dptile);
  sl::splitk_scratch() = sl::SplitKScratch();
  if (g_dev.stream) cudaStreamDestroy(g_dev.stream);
  if (g_dev.aux) cudaStreamDestroy(g_dev.aux);
  if (g_dev.ev_next) cudaEventDestroy(g_dev.ev_next);
  if (g_dev.ev_panel) cudaEventDestroy(g_dev.ev_panel);
  if (g_dev.h2d) cudaStreamDestroy(g_dev.h2d);
  if (g_dev.ev_h2d) cudaEventDestroy(g_dev.ev_h2d);
  for (cudaEvent_t ev : g_dev.ev_cols)
    if (ev) cudaEventDestroy(ev);
  g_dev = DevState();
}

// Grows a sliced-product scratch buffer; a new one starts with its balancing
// words zeroed (the memory may hold anything, including words that look like
// a later epoch's).
static cudaError_t grow_oz(unsigned char** p, size_t* cap, size_t need) {
  const unsigned char* old = *p;
  cudaError_t e = grow(p, cap, need);
  if (e == cudaSuccess && *p != old)
    e = cudaMemset(*p, 0, *cap < (size_t)sl::kOzKinfoBytes ? *cap : (size_t)sl::kOzKinfoBytes);
  return e;
}

void ensure_oz(int m, int n, int nb) {
  // panels taller than the SMs' shared memory holds keep their rows in a
  // global buffer (optional: without it such an M is rejected with -30000)
  if (m > sl::panel_max_rows() && n > 0 &&
      grow(&g_dev.dptile, &g_dev.capPtile, sl::panel_tile_doubles(m)) != cudaSuccess)
    cudaGetLastError();
  if (sl::f64_update_get() != 1 || m <= 0 || n <= 0) return;
  if (nb <= 0) nb = g_default_nb;
  const size_t need = sl::oz_scratch_bytes(m, n, nb);
  // the panel's 32-column updates and the next panel's columns (nb x nb)
  const size_t need2 = sl::oz_scratch_bytes(m, nb, nb > 32 ? nb : 32);
  cudaError_t e = cudaSuccess;
  if (need > g_dev.capOz || !g_dev.doz) e = grow_oz(&g_dev.doz, &g_dev.capOz, need);
  if (e == cudaSuccess && (need2 > g_dev.capOz2 || !g_dev.doz2))
    e = grow_oz(&g_dev.doz2, &g_dev.capOz2, need2);
  if (e == cudaSuccess && !g_dev.ddinv64)
    e = cudaMalloc(&g_dev.ddinv64, 3 * sl::kDinv64Doubles * sizeof(double));
  if (e != cudaSuccess) cudaGetLastError();  // the DMMA update covers what is missing
}

sl::LuWork make_work() {
  sl::LuWork w;
  w.status = g_dev.dsmall + 2;
  w.info_col = g_dev.dsmall + 3;
  w.cand = g_dev.dcand;
  w.swap_plan = g_dev.dplan;
  w.perm = g_dev.dperm;
  w.bswap = g_dev.dbswap;
  w.perm_len = g_dev.capPerm;
  w.bswap_len = g_dev.capBs;
  w.oz.ptr = g_dev.doz;
  w.oz.bytes = g_dev.doz ? g_dev.capOz : 0;
  w.oz_aux.ptr = g_dev.doz2;
  w.oz_aux.bytes = g_dev.doz2 ? g_dev.capOz2 : 0;
  w.dinv64 = g_dev.ddinv64;
  w.dinv64_step0 = g_dev.ddinv64 ? g_dev.ddinv64 + sl::kDinv64Doubles : nullptr;
  w.dinv64_alt = (g_dev.ddinv64 && g_split_step) ? g_dev.ddinv64 + 2 * sl::kDinv64Doubles : nullptr;
  w.swap_plan_alt = g_split_step ? g_dev.dplan + sl::kSwapPlanInts : nullptr;
  w.dinv_solve = g_dev.ddinvs;
  w.dinv_solve_len = g_dev.ddinvs ? g_dev.capDinvs : 0;
  w.ptile = g_dev.dptile;
  w.ptile_len = g_dev.dptile ? g_dev.capPtile : 0;
  if (g_lookahead) {
    w.aux = g_dev.aux;
    w.ev_next = g_dev.ev_next;
    w.ev_panel = g_dev.ev_panel;
  }
  return w;
}

cudaError_t ensure_solve_ws(int n, int nrhs) {
  cudaError_t e = grow(&g_dev.dperm, &g_dev.capPerm, (size_t)n);
  if (e != cudaSuccess) return e;
  e = grow(&g_dev.dbswap, &g_dev.capBs, (size_t)n * (size_t)nrhs);
  if (e != cudaSuccess) return e;
  if (sl::f64_update_get() == 1) {
    // blocked solve with diagonal-block inverses and sliced updates (optional:
    // without them the substitution solves run)
    ensure_oz(n, nrhs, 128);
    if (grow(&g_dev.ddinvs, &g_dev.capDinvs, sl::kSolveInvDoubles(n)) != cudaSuccess) cudaGetLastError();
  }
  return cudaSuccess;
}

// Reads the device status word and the first zero-pivot column after a
// factorization; returns INFO (>0 singular, <=-20000 device status).
int read_factor_info(cudaStream_t s, int mn, int* out_info) {
  int h[2] = {0, 0};
  cudaError_t e = cudaMemcpyAsync(h, g_dev.dsmall + 2, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { *out_info = cuda_info(e); return *out_info; }
  if (h[0] != 0) { *out_info = -20000 - h[0]; return *out_info; }
  *out_info = (h[1] >= 0 && h[1] < mn) ? h[1] + 1 : 0;
  return *out_info;
}

long long round_ld(long long m) {
  long long ld = m < 1 ? 1 : m;
  return (ld + 31) / 32 * 32;
}

// ---- shared implementation of the host-ABI entry points ---------------------
// With copy_stream set, the factors' copy back to A is only issued there (the
// caller synchronizes it later, e.g. after running the solve beside it);
// IPIV and INFO are always complete on return.
int factor_host(int m, int n, double* A, int ia, int ja, const int* desca, int* ipiv,
                cudaStream_t s, long long* ldda_out, cudaStream_t copy_stream) {
  const long long lld = desca[LLD_];
  const long long ldda = round_ld(m);
  const int mn = m < n ? m : n;
  cudaError_t e = grow(&g_dev.dA, &g_dev.capA, (size_t)ldda * (size_t)n);
  if (e == cudaSuccess) e = grow(&g_dev.dipiv, &g_dev.capP, (size_t)(mn > 0 ? mn : 1));
  if (e != cudaSuccess) return cuda_info(e);
  const double* src = A + (ia - 1) + (long long)(ja - 1) * lld;
  ensure_oz(m, n, desca[NB_]);
  // With the look-ahead on and more than two panels, A goes over in column
  // chunks of about n/g_copy_chunks (whole panels, the first holding panels 0
  // and 1) on the copy stream, and step 0 of the factorization follows them.
  const int nbk = desca[NB_] < 1024 ? desca[NB_] : 1024;
  int col_end[sl::kMaxColChunks];
  int nck = 0;
  if (g_copy_chunks > 1 && g_lookahead && nbk > 0 && mn > 2 * nbk) {
    const long long per = ((long long)n + g_copy_chunks - 1) / g_copy_chunks;
    long long w = (per + nbk - 1) / nbk * nbk;
    if (w < 2LL * nbk) w = 2LL * nbk;
    e = cudaEventRecord(g_dev.ev_h2d, s);  // dA is free once s's earlier work is done
    if (e == cudaSuccess) e = cudaStreamWaitEvent(g_dev.h2d, g_dev.ev_h2d, 0);
    for (long long a = 0; e == cudaSuccess && a < n; a += w) {
      const long long b = (a + w >= n || nck == sl::kMaxColChunks - 1) ? n : a + w;
      e = cudaMemcpy2DAsync(g_dev.dA + a * ldda, ldda * sizeof(double), src + a * lld,
                            lld * sizeof(double), (size_t)m * sizeof(double), (size_t)(b - a),
                            cudaMemcpyHostToDevice, g_dev.h2d);
      if (e == cudaSuccess) e = cudaEventRecord(g_dev.ev_cols[nck], g_dev.h2d);
      col_end[nck++] = (int)b;
      if (b == n) break;
    }
    if (e != cudaSuccess) {
      cudaStreamSynchronize(g_dev.h2d);
      return cuda_info(e);
    }
  } else {
    e = cudaMemcpy2DAsync(g_dev.dA, ldda * sizeof(double), src, lld * sizeof(double),
                          (size_t)m * sizeof(double), n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_info(e);
  }
  sl::LuWork w = make_work();
  w.ncol_chunks = nck;
  w.col_end = col_end;
  w.ev_cols = g_dev.ev_cols;
  e = sl::dgetrf_device(m, n, g_dev.dA, ldda, g_dev.dipiv, desca[NB_], w, s);
  // (every chunk has been waited for on s unless the factorization stopped early)
  if (nck > 0) {
    const cudaError_t e2 = cudaStreamSynchronize(g_dev.h2d);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaErrorInvalidValue) return -30000;
  if (e != cudaSuccess) return cuda_info(e);
  int info = 0;
  read_factor_info(s, mn, &info);
  if (info <= -10000) return info;
  // copy the pivots and factors back: IPIV(IA+k) = IA + p (global 1-based row);
  // the factorization is complete (read_factor_info synchronized s). The
  // pivots come first: a small device-to-host copy issued after the factors'
  // would wait behind them for the copy engine, and so would the caller's
  // solve on s.
  std::vector<int> hp((size_t)(mn > 0 ? mn : 1));
  e = cudaMemcpyAsync(hp.data(), g_dev.dipiv, (size_t)mn * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(A + (ia - 1) + (long long)(ja - 1) * lld, lld * sizeof(double), g_dev.dA,
                          ldda * sizeof(double), (size_t)m * sizeof(double), n,
                          cudaMemcpyDeviceToHost, copy_stream ? copy_stream : s);
  if (e == cudaSuccess && !copy_stream) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_info(e);
  for (int k = 0; k < mn; ++k) ipiv[ia - 1 + k] = ia + hp[k];
  if (ldda_out) *ldda_out = ldda;
  return info;
}

int validate_getrf(const char* name, int m, int n, int ia, int ja, const int* desca) {
  int nprow, npcol, myrow, mycol;
  gridinfo(desca[CTXT_], &nprow, &npcol, &myrow, &mycol);
  int info = 0;
  if (nprow == -1) {
    info = -(600 + FCTXT);
  } else {
    chk1mat(m, 1, n, 2, ia, ja, desca, 6, &info);
    if (info == 0) {
      int iroff = (ia - 1) % desca[MB_], icoff = (ja - 1) % desca[NB_];
      if (iroff != 0) info = -4;
      else if (icoff != 0) info = -5;
      else if (desca[MB_] != desca[NB_]) info = -(600 + FNB);
    }
  }
  if (info != 0) pxerbla(desca[CTXT_], name, -info);
  return info;
}

}  // namespace host
}  // namespace sl

using namespace sl::host;

namespace sl {
int default_nb() { return host::g_default_nb; }
}  // namespace sl

extern "C" {

// ---------------------------------------------------------------- PDGETRF
void pdgetrf_(const int* M, const int* N, double* A, const int* IA, const int* JA,
              const int* DESCA, int* IPIV, int* INFO) {
  std::lock_guard<std::mutex> lk(g_mu);
  *INFO = validate_getrf("PDGETRF", *M, *N, *IA, *JA, DESCA);
  if (*INFO != 0) return;
  // Quick return (SRC/pdgetrf.f:201-206): tests the global M_A.
  if (DESCA[M_] == 1) { IPIV[0] = 1; return; }
  if (*M == 0 || *N == 0) return;
  if (!ensure_device()) { *INFO = cuda_info(cudaErrorNoDevice); return; }
  *INFO = factor_host(*M, *N, A, *IA, *JA, DESCA, IPIV, g_dev.stream, nullptr, nullptr);
}

// ---------------------------------------------------------------- PDGETRS
static int validate_getrs(char trans, int n, int nrhs, int ia, int ja, const int* desca, int ib,
                          int jb, const int* descb) {
  int nprow, npcol, myrow, mycol;
  gridinfo(desca[CTXT_], &nprow, &npcol, &myrow, &mycol);
  int info = 0;
  if (nprow == -1) {
    info = -(700 + FCTXT);
  } else {
    bool notran = (trans == 'N' || trans == 'n');
    chk1mat(n, 2, n, 2, ia, ja, desca, 7, &info);
    chk1mat(n, 2, nrhs, 3, ib, jb, descb, 12, &info);
    if (info == 0) {
      int iroffa = (ia - 1) % desca[MB_], icoffa = (ja - 1) % desca[NB_];
      int iroffb = (ib - 1) % descb[MB_];
      // INDXG2P is 0 for both on a 1x1 grid, so IBROW == IAROW.
      if (!notran && !(trans == 'T' || trans == 't') && !(trans == 'C' || trans == 'c')) info = -1;
      else if (iroffa != 0) info = -5;
      else if (icoffa != 0) info = -6;
      else if (desca[MB_] != desca[NB_]) info = -(700 + FNB);
      else if (iroffb != 0) info = -10;
      else if (descb[MB_] != desca[NB_]) info = -(1200 + FNB);
      else if (desca[CTXT_] != descb[CTXT_]) info = -(1200 + FCTXT);
    }
  }
  if (info != 0) pxerbla(desca[CTXT_], "PDGETRS", -info);
  return info;
}

static int solve_host(char trans, int n, int nrhs, long long ldda, double* B, int ib, int jb,
                      const int* descb, cudaStream_t s) {
  const long long lldb = descb[LLD_];
  const long long lddb = round_ld(n);
  cudaError_t e = grow(&g_dev.dB, &g_dev.capB, (size_t)lddb * (size_t)nrhs);
  if (e == cudaSuccess) e = ensure_solve_ws(n, nrhs);
  if (e != cudaSuccess) return cuda_info(e);
  double* hb = B + (ib - 1) + (long long)(jb - 1) * lldb;
  e = cudaMemcpy2DAsync(g_dev.dB, lddb * sizeof(double), hb, lldb * sizeof(double),
                        (size_t)n * sizeof(double), nrhs, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_info(e);
  sl::LuWork w = make_work();
  e = sl::dgetrs_device(trans, n, nrhs, g_dev.dA, ldda, g_dev.dipiv, g_dev.dB, lddb, w, s);
  if (e != cudaSuccess) return cuda_info(e);
  e = cudaMemcpy2DAsync(hb, lldb * sizeof(double), g_dev.dB, lddb * sizeof(double),
                        (size_t)n * sizeof(double), nrhs, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_info(e);
  return 0;
}

void pdgetrs_(const char* TRANS, const int* N, const int* NRHS, const double* A, const int* IA,
              const int* JA, const int* DESCA, const int* IPIV, double* B, const int* IB,
              const int* JB, const int* DESCB, int* INFO, size_t TRANS_len) {
  (void)TRANS_len;
  std::lock_guard<std::mutex> lk(g_mu);
  const char trans = TRANS[0];
  *INFO = validate_getrs(trans, *N, *NRHS, *IA, *JA, DESCA, *IB, *JB, DESCB);
  if (*INFO != 0) return;
  if (*N == 0 || *NRHS == 0) return;
  if (!ensure_device()) { *INFO = cuda_info(cudaErrorNoDevice); return; }
  const int n = *N, ia = *IA, ja = *JA;
  const long long lld = DESCA[LLD_];
  const long long ldda = round_ld(n);
  cudaStream_t s = g_dev.stream;
  cudaError_t e = grow(&g_dev.dA, &g_dev.capA, (size_t)ldda * (size_t)n);
  if (e == cudaSuccess) e = grow(&g_dev.dipiv, &g_dev.capP, (size_t)n);
  if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  e = cudaMemcpy2DAsync(g_dev.dA, ldda * sizeof(double), A + (ia - 1) + (long long)(ja - 1) * lld,
                        lld * sizeof(double), (size_t)n * sizeof(double), n,
                        cudaMemcpyHostToDevice, s);
  // IPIV holds global 1-based rows; the device path wants rows relative to IA.
  std::vector<int> hp((size_t)n);
  for (int k = 0; k < n; ++k) hp[k] = IPIV[ia - 1 + k] - ia;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g_dev.dipiv, hp.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  *INFO = solve_host(trans, n, *NRHS, ldda, B, *IB, *JB, DESCB, s);
}

// ---------------------------------------------------------------- PDGESV
void pdgesv_(const int* N, const int* NRHS, double* A, const int* IA, const int* JA,
             const int* DESCA, int* IPIV, double* B, const int* IB, const int* JB,
             const int* DESCB, int* INFO) {
  std::lock_guard<std::mutex> lk(g_mu);
  int nprow, npcol, myrow, mycol;
  gridinfo(DESCA[CTXT_], &nprow, &npcol, &myrow, &mycol);
  int info = 0;
  const int n = *N, nrhs = *NRHS, ia = *IA, ja = *JA, ib = *IB, jb = *JB;
  if (nprow == -1) {
    info = -(600 + FCTXT);
  } else {
    chk1mat(n, 1, n, 1, ia, ja, DESCA, 6, &info);
    chk1mat(n, 1, nrhs, 2, ib, jb, DESCB, 11, &info);
    if (info == 0) {
      int iroffa = (ia - 1) % DESCA[MB_], icoffa = (ja - 1) % DESCA[NB_];
      int iroffb = (ib - 1) % DESCB[MB_];
      if (iroffa != 0) info = -4;
      else if (icoffa != 0) info = -5;
      else if (DESCA[MB_] != DESCA[NB_]) info = -(600 + FNB);
      else if (icoffa != iroffb) info = -9;
      else if (DESCB[MB_] != DESCA[NB_]) info = -(1100 + FNB);
      else if (DESCA[CTXT_] != DESCB[CTXT_]) info = -(1100 + FCTXT);
    }
  }
  if (info != 0) {
    pxerbla(DESCA[CTXT_], "PDGESV", -info);
    *INFO = info;
    return;
  }
  // PDGETRF (SRC/pdgesv.f:229) -- its own validation cannot fail here.
  *INFO = 0;
  if (DESCA[M_] == 1) IPIV[0] = 1;
  if (n == 0) return;
  if (!ensure_device()) { *INFO = cuda_info(cudaErrorNoDevice); return; }
  long long ldda = round_ld(n);
  if (DESCA[M_] == 1) {
    // 1x1 global matrix: PDGETRF returns at once with IPIV(1) = 1 and INFO = 0,
    // so PDGETRS runs on the unfactored 1x1 A.
    cudaStream_t s = g_dev.stream;
    cudaError_t e = grow(&g_dev.dA, &g_dev.capA, (size_t)ldda);
    if (e == cudaSuccess) e = grow(&g_dev.dipiv, &g_dev.capP, 1);
    int zero = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(g_dev.dA, A + (ia - 1) + (long long)(ja - 1) * DESCA[LLD_], sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g_dev.dipiv, &zero, sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  } else {
    // the factors go back to A on the second stream while the solve runs
    *INFO = factor_host(n, n, A, ia, ja, DESCA, IPIV, g_dev.stream, &ldda, g_dev.aux);
  }
  auto join_copy = [&]() {
    if (DESCA[M_] != 1) {
      cudaError_t e = cudaStreamSynchronize(g_dev.aux);
      if (e != cudaSuccess && *INFO == 0) *INFO = cuda_info(e);
    }
  };
  if (*INFO != 0 || nrhs == 0) {  // singular (or GPU failure): the solve is skipped (pdgesv.f:231)
    join_copy();
    return;
  }
  *INFO = solve_host('N', n, nrhs, ldda, B, ib, jb, DESCB, g_dev.stream);
  join_copy();
}

// ---------------------------------------------------------------- TOOLS
int numroc_(const int* N, const int* NB, const int* IPROC, const int* ISRCPROC, const int* NPROCS) {
  return numroc(*N, *NB, *IPROC, *ISRCPROC, *NPROCS);
}

void descinit_(int* DESC, const int* M, const int* N, const int* MB, const int* NB,
               const int* IRSRC, const int* ICSRC, const int* ICTXT, const int* LLD, int* INFO) {
  // TOOLS/descinit.f:148-192
  int nprow, npcol, myrow, mycol;
  int c = *ICTXT;
  blacs_gridinfo_(&c, &nprow, &npcol, &myrow, &mycol);
  int info = 0;
  if (*M < 0) info = -2;
  else if (*N < 0) info = -3;
  else if (*MB < 1) info = -4;
  else if (*NB < 1) info = -5;
  else if (*IRSRC < 0 || *IRSRC >= nprow) info = -6;
  else if (*ICSRC < 0 || *ICSRC >= npcol) info = -7;
  else if (nprow == -1) info = -8;
  else {
    int lr = numroc(*M, *MB, myrow, *IRSRC, nprow);
    if (*LLD < (lr > 1 ? lr : 1)) info = -9;
  }
  if (info != 0) pxerbla(*ICTXT, "DESCINIT", -info);
  auto mx = [](int a, int b) { return a > b ? a : b; };
  auto mnf = [](int a, int b) { return a < b ? a : b; };
  DESC[DTYPE_] = 1;
  DESC[M_] = mx(0, *M);
  DESC[N_] = mx(0, *N);
  DESC[MB_] = mx(1, *MB);
  DESC[NB_] = mx(1, *NB);
  DESC[RSRC_] = mx(0, mnf(*IRSRC, nprow - 1));
  DESC[CSRC_] = mx(0, mnf(*ICSRC, npcol - 1));
  DESC[CTXT_] = *ICTXT;
  int lr = (nprow > 0) ? numroc(DESC[M_], DESC[MB_], myrow, DESC[RSRC_], nprow) : 1;
  DESC[LLD_] = mx(*LLD, mx(1, lr));
  *INFO = info;
}

// ---------------------------------------------------------------- BLACS shim
void blacs_pinfo_(int* MYPNUM, int* NPROCS) { *MYPNUM = 0; *NPROCS = 1; }

void blacs_get_(const int* ICTXT, const int* WHAT, int* VAL) {
  (void)ICTXT;
  // WHAT = 0 (SGET_SYSCONTXT) and 10 (SGET_BLACSCONTXT) return the system
  // context handle, which is 0 for the single process.
  if (*WHAT == 0 || *WHAT == 10) *VAL = 0;
  else *VAL = 0;
}

void blacs_gridinit_(int* ICTXT, const char* ORDER, const int* NPROW, const int* NPCOL,
                     size_t ORDER_len) {
  (void)ORDER; (void)ORDER_len;
  std::lock_guard<std::mutex> lk(g_grid_mu);
  Grid g;
  g.live = true;
  g.nprow = *NPROW;
  g.npcol = *NPCOL;
  g_grids.push_back(g);
  *ICTXT = (int)g_grids.size() - 1;
}

void blacs_gridinfo_(const int* ICTXT, int* NPROW, int* NPCOL, int* MYROW, int* MYCOL) {
  shim_gridinfo(*ICTXT, NPROW, NPCOL, MYROW, MYCOL);
}

void blacs_gridexit_(const int* ICTXT) {
  std::lock_guard<std::mutex> lk(g_grid_mu);
  if (*ICTXT >= 0 && *ICTXT < (int)g_grids.size()) g_grids[*ICTXT].live = false;
}

void blacs_exit_(const int* CONTINUE) {
  (void)CONTINUE;
  {
    std::lock_guard<std::mutex> lk(g_grid_mu);
    for (auto& g : g_grids) g.live = false;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  release_all();
}

// ------------------------------------------------------- device entry points
int sl1x1_dgetrf_dev(int m, int n, double* dA, long long ldda, int* dipiv, int nb, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (ldda < (m > 1 ? m : 1)) return -4;
  if (m == 0 || n == 0) return 0;
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  cudaStream_t s = (cudaStream_t)stream;
  if (nb <= 0) nb = g_default_nb;
  ensure_oz(m, n, nb);
  sl::LuWork w = make_work();
  cudaError_t e = sl::dgetrf_device(m, n, dA, ldda, dipiv, nb, w, s);
  if (e == cudaErrorInvalidValue) return -30000;
  if (e != cudaSuccess) return cuda_info(e);
  int mn = m < n ? m : n;
  int info = 0;
  read_factor_info(s, mn, &info);
  if (info <= -10000) return info;
  e = sl::ipiv_shift(dipiv, dipiv, mn, 1, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_info(e);
  return info;
}

int sl1x1_dgetrs_dev(char trans, int n, int nrhs, const double* dA, long long ldda,
                     const int* dipiv, double* dB, long long lddb, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  bool ok_t = trans == 'N' || trans == 'n' || trans == 'T' || trans == 't' || trans == 'C' ||
              trans == 'c';
  if (!ok_t) return -1;
  if (n < 0) return -2;
  if (nrhs < 0) return -3;
  if (ldda < (n > 1 ? n : 1)) return -5;
  if (lddb < (n > 1 ? n : 1)) return -8;
  if (n == 0 || nrhs == 0) return 0;
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = grow(&g_dev.dipiv, &g_dev.capP, (size_t)n);
  if (e == cudaSuccess) e = ensure_solve_ws(n, nrhs);
  if (e != cudaSuccess) return cuda_info(e);
  e = sl::ipiv_shift(dipiv, g_dev.dipiv, n, -1, s);
  if (e != cudaSuccess) return cuda_info(e);
  sl::LuWork w = make_work();
  e = sl::dgetrs_device(trans, n, nrhs, dA, ldda, g_dev.dipiv, dB, lddb, w, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_info(e);
  return 0;
}

int sl1x1_dgesv_dev(int n, int nrhs, double* dA, long long ldda, int* dipiv, double* dB,
                    long long lddb, int nb, void* stream) {
  int info = sl1x1_dgetrf_dev(n, n, dA, ldda, dipiv, nb, stream);
  if (info != 0) return info;
  return sl1x1_dgetrs_dev('N', n, nrhs, dA, ldda, dipiv, dB, lddb, stream);
}

int sl1x1_lowp_update_dev(int fmt, int m, int n, int k, const float* dL, long long ldl,
                          const float* dU, long long ldu, float* dC, long long ldc, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (fmt < 0 || fmt > 2) return -1;
  if (m < 0) return -2;
  if (n < 0) return -3;
  if (k < 0) return -4;
  if (m == 0 || n == 0 || k == 0) return 0;
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  cudaStream_t s = (cudaStream_t)stream;
  const int kpad = sl::lowp_kpad(k) * sl::lowp_kmult(fmt);
  cudaError_t e = grow(&g_dev.dA16, &g_dev.capA16, (size_t)m * kpad);
  if (e == cudaSuccess) e = grow(&g_dev.dB16, &g_dev.capB16, (size_t)n * kpad);
  if (e == cudaSuccess) e = grow(&g_dev.dcolexp, &g_dev.capCe, (size_t)n);
  if (e != cudaSuccess) return cuda_info(e);
  e = cudaMemsetAsync(g_dev.dsmall + 2, 0, sizeof(int), s);
  if (e == cudaSuccess)
    e = sl::lowp_pack(fmt, dL, ldl, m, dU, ldu, n, k, g_dev.dA16, g_dev.dB16, g_dev.dcolexp, s);
  if (e == cudaSuccess)
    e = sl::lowp_gemm(fmt, m, n, k, g_dev.dA16, g_dev.dB16, g_dev.dcolexp, dC, ldc,
                      g_dev.dsmall + 2, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_info(e);
  int st = 0;
  e = cudaMemcpy(&st, g_dev.dsmall + 2, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_info(e);
  return st ? -20000 - st : 0;
}

int sl1x1_dgesv_ir_dev(int n, int nrhs, double* dA, long long ldda, int* dipiv, const double* dB,
                       long long lddb, double* dX, long long lddx, int fmt, int nb, double tol,
                       int keep_a, int* iter, double* stats, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (n < 0) return -1;
  if (nrhs < 0) return -2;
  if (ldda < (n > 1 ? n : 1)) return -4;
  if (lddb < (n > 1 ? n : 1)) return -7;
  if (lddx < (n > 1 ? n : 1)) return -9;
  if (fmt < 0 || fmt > 2) return -10;
  if (iter) *iter = 0;
  if (n == 0 || nrhs == 0) return 0;
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  cudaStream_t s = (cudaStream_t)stream;
  sl::IrOptions opt;
  opt.fmt = fmt;
  opt.nb = nb > 0 ? nb : 256;
  opt.nb_fp64 = g_default_nb;
  if (tol > 0) opt.tol = tol;
  opt.fp64_cost_ratio = g_ir_cost_ratio;
  ensure_oz(n, n, opt.nb_fp64);  // the FP64 fallback factorization
  const long long ldf = round_ld(n);
  const int kpad = sl::lowp_kpad(opt.nb) * sl::lowp_kmult(fmt);
  const size_t m1 = (size_t)opt.gmres_m + 1;
  cudaError_t e = cudaSuccess;
#define GROW(p, c, cnt) if (e == cudaSuccess) e = grow(&g_dev.p, &g_dev.c, (size_t)(cnt))
  GROW(dF, capF, (size_t)ldf * n);
  GROW(dA16, capA16, (size_t)n * kpad);
  GROW(dB16, capB16, (size_t)n * kpad);
  GROW(dcolexp, capCe, n);
  GROW(dpermx, capPermx, n);
  GROW(dR, capR, (size_t)n * nrhs);
  GROW(dD, capD, n);
  GROW(dXf, capXf, (size_t)n * nrhs);
  GROW(dXt, capXt, (size_t)n * nrhs);
  GROW(dcm, capCm, 2 * (size_t)nrhs + 8);
  GROW(dV, capV, (size_t)n * m1);
  GROW(dw, capW, n);
  GROW(dAx, capAx, n);
  GROW(dh, capH, m1 + 8);
  GROW(dperm, capPerm, n);
  GROW(dbswap, capBs, (size_t)n * nrhs);
  if (keep_a) GROW(dAcopy, capAcopy, (size_t)ldf * n);
  GROW(dsplitk, capSplitk, (size_t)32 * 4 * n);  // split-K partials of the FP64 products
  GROW(ddinv, capDinv, (size_t)4 * ((n + 63) / 64) * 64 * 64);  // diagonal-block inverses and M_b
  // mirror the buffer whatever happened above: a failed grow freed it (null,
  // capacity 0), and a stale pointer here would reach every later split-K
  // product
  sl::splitk_scratch().ptr = g_dev.dsplitk;
  sl::splitk_scratch().bytes = g_dev.capSplitk * sizeof(double);
  {
    // ticket (64 bytes) + n x 8 values of the chained solves, each up to two
    // tagged 8-byte words (FP64 vectors)
    const size_t need = 16 + (size_t)n * 8 * 2 * 2;
    if (need > g_dev.capChain || !g_dev.dchain) {
      GROW(dchain, capChain, need);
      if (e == cudaSuccess) e = cudaMemsetAsync(g_dev.dchain, 0, sizeof(int) * g_dev.capChain, s);
      g_dev.chain_epoch = 0;  // fresh flags
    }
  }
#undef GROW
  if (e != cudaSuccess) return cuda_info(e);
  sl::MixedWork mw;
  mw.F = g_dev.dF; mw.ldf = ldf;
  mw.A16 = g_dev.dA16; mw.B16 = g_dev.dB16; mw.col_exp = g_dev.dcolexp;
  mw.perm = g_dev.dpermx; mw.R = g_dev.dR; mw.D = g_dev.dD;
  mw.Xf = g_dev.dXf; mw.Xtmp = g_dev.dXt; mw.colmax = g_dev.dcm;
  mw.V = g_dev.dV; mw.w = g_dev.dw; mw.Ax = g_dev.dAx; mw.h = g_dev.dh;
  mw.Acopy = keep_a ? g_dev.dAcopy : nullptr; mw.ldacopy = ldf;
  mw.chain = g_dev.dchain; mw.epoch = &g_dev.chain_epoch; mw.status = g_dev.dsmall + 4;
  mw.dinv = g_dev.ddinv;
  if (e == cudaSuccess) e = cudaMemsetAsync(mw.status, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_info(e);
  sl::LuWork w = make_work();
  sl::IrStats st;
  e = sl::dgesv_ir_device(n, nrhs, dA, ldda, dB, lddb, dX, lddx, g_dev.dipiv == nullptr ? dipiv : dipiv,
                          opt, &st, w, mw, s);
  if (e == cudaErrorInvalidValue) return -30000;
  if (e != cudaSuccess) return cuda_info(e);
  if (stats) {
    stats[0] = st.classical; stats[1] = st.gmres_outer; stats[2] = st.gmres_inner;
    stats[3] = st.fell_back ? (st.gave_up ? 2 : 1) : 0; stats[4] = st.sresid; stats[5] = st.anorm;
    stats[6] = st.factor_ms; stats[7] = st.refine_ms;
  }
  if (st.dev_status) return -20000 - st.dev_status;
  if (iter) *iter = st.fell_back ? (st.gmres_outer > 0 || st.classical > 0 ? -3 : -1)
                                 : st.classical + st.gmres_outer;
  return st.info;
}

int sl1x1_batch_plan_create(sl1x1_batch_plan* plan, int batch, const int* n, const int* nrhs,
                            const double* const* dA, const int* lda, const double* const* dB,
                            const int* ldb, double* const* dX, const int* ldx, int mode, double tol,
                            int autotune, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!plan) return -1;
  *plan = nullptr;
  if (batch < 0) return -2;
  for (int i = 0; i < batch; ++i) {
    if (n[i] < 1 || n[i] > 512) return -3;
    if (nrhs[i] < 1 || nrhs[i] > 8) return -4;
    if (lda[i] < n[i]) return -6;
    if (ldb[i] < n[i]) return -8;
    if (ldx[i] < n[i]) return -10;
  }
  if (mode != 0 && mode != 1) return -11;
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  sl::BatchPlan* p = nullptr;
  cudaError_t e = sl::batch_plan_create(&p, batch, n, nrhs, dA, lda, dB, ldb, dX, ldx, mode, tol,
                                        autotune, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_info(e);
  *plan = reinterpret_cast<sl1x1_batch_plan>(p);
  return 0;
}

int sl1x1_batch_plan_execute(sl1x1_batch_plan plan, void* stream) {
  if (!plan) return -1;
  cudaError_t e = sl::batch_plan_execute(reinterpret_cast<sl::BatchPlan*>(plan), (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  return e == cudaSuccess ? 0 : cuda_info(e);
}

int sl1x1_batch_plan_results(sl1x1_batch_plan plan, int* info, int* iters, double* sresid,
                             void* stream) {
  if (!plan) return -1;
  cudaError_t e = sl::batch_plan_results(reinterpret_cast<sl::BatchPlan*>(plan), info, iters,
                                         sresid, (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : cuda_info(e);
}

int sl1x1_batch_plan_shape(sl1x1_batch_plan plan, int* threads, int* chunk, int* ctas_per_sm) {
  if (!plan) return -1;
  sl::batch_plan_shape(reinterpret_cast<sl::BatchPlan*>(plan), threads, chunk, ctas_per_sm);
  return 0;
}

void sl1x1_batch_plan_destroy(sl1x1_batch_plan plan) {
  sl::batch_plan_destroy(reinterpret_cast<sl::BatchPlan*>(plan));
}

// ------------------------------------------------------ norms / rcond / inverse
static char upc(char c) { return (c >= 'a' && c <= 'z') ? (char)(c - 32) : c; }

double sl1x1_dlange_dev(char norm, int m, int n, const double* dA, long long ldda, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (m <= 0 || n <= 0) return 0.0;
  if (!ensure_device()) return NAN;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = grow(&g_dev.daux, &g_dev.capAux, (size_t)(m > n ? m : n) + 8);
  double v = NAN;
  if (e == cudaSuccess)
    e = sl::dlange_device(norm, m, n, dA, ldda, g_dev.daux, g_dev.daux + (m > n ? m : n) + 4, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&v, g_dev.daux + (m > n ? m : n) + 4, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "sl1x1_dlange_dev: CUDA error %d\n", (int)e);
    return NAN;
  }
  return v;
}

// PDLANGE (SRC/pdlange.f:1): the norm of sub(A), computed on the GPU.
double pdlange_(const char* NORM, const int* M, const int* N, const double* A, const int* IA,
                const int* JA, const int* DESCA, double* WORK, size_t NORM_len) {
  (void)WORK; (void)NORM_len;
  const int m = *M, n = *N;
  if (m <= 0 || n <= 0) return 0.0;
  double* dA = nullptr;
  long long ldda = 0;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!ensure_device()) {
      std::fprintf(stderr, "pdlange_: no usable sm_103 GPU\n");
      return NAN;
    }
    ldda = round_ld(m);
    if (grow(&g_dev.dA, &g_dev.capA, (size_t)ldda * n) != cudaSuccess) return NAN;
    const long long lld = DESCA[LLD_];
    if (cudaMemcpy2DAsync(g_dev.dA, ldda * sizeof(double), A + (*IA - 1) + (long long)(*JA - 1) * lld,
                          lld * sizeof(double), (size_t)m * sizeof(double), n,
                          cudaMemcpyHostToDevice, g_dev.stream) != cudaSuccess)
      return NAN;
    dA = g_dev.dA;
  }
  return sl1x1_dlange_dev(NORM[0], m, n, dA, ldda, g_dev.stream);
}

int sl1x1_dgecon_dev(char norm, int n, const double* dLU, long long ldda, double anorm,
                     double* rcond, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  const char u = upc(norm);
  const bool onenrm = (u == '1' || u == 'O');
  if (!onenrm && u != 'I') return -1;
  if (n < 0) return -2;
  if (ldda < (n > 1 ? n : 1)) return -4;
  if (anorm < 0.0) return -5;
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = grow(&g_dev.daux, &g_dev.capAux, 3 * (size_t)n + 16);
  if (e != cudaSuccess) return cuda_info(e);
  e = sl::dgecon_device(onenrm, n, dLU, ldda, anorm, rcond, g_dev.daux,
                        reinterpret_cast<int*>(g_dev.daux + 3 * (size_t)n + 8), s);
  return e == cudaSuccess ? 0 : cuda_info(e);
}

// PDGECON (SRC/pdgecon.f): validation, workspace query and quick returns as
// the reference; the estimate is computed on the GPU from the LU factors.
void pdgecon_(const char* NORM, const int* N, const double* A, const int* IA, const int* JA,
              const int* DESCA, const double* ANORM, double* RCOND, double* WORK,
              const int* LWORK, int* IWORK, const int* LIWORK, int* INFO, size_t NORM_len) {
  (void)NORM_len;
  int nprow, npcol, myrow, mycol;
  gridinfo(DESCA[CTXT_], &nprow, &npcol, &myrow, &mycol);
  int info = 0;
  const int n = *N, ia = *IA, ja = *JA;
  const char u = upc(NORM[0]);
  const bool onenrm = (NORM[0] == '1' || u == 'O');
  bool lquery = false;
  if (nprow == -1) {
    info = -(600 + FCTXT);
  } else {
    chk1mat(n, 2, n, 2, ia, ja, DESCA, 6, &info);
    if (info == 0) {
      const int npmod = numroc(n + (ia - 1) % DESCA[MB_], DESCA[MB_], 0, 0, 1);
      const int nqmod = numroc(n + (ja - 1) % DESCA[NB_], DESCA[NB_], 0, 0, 1);
      const int nb = DESCA[NB_];
      int inner = nb > nqmod + nb ? nb : nqmod + nb;
      const int lwmin = 2 * npmod + 2 * nqmod + (inner > 2 ? inner : 2);
      const int liwmin = npmod > 1 ? npmod : 1;
      WORK[0] = (double)lwmin;
      IWORK[0] = liwmin;
      lquery = (*LWORK == -1 || *LIWORK == -1);
      if (!onenrm && u != 'I') info = -1;
      else if (*ANORM < 0.0) info = -7;
      else if (*LWORK < lwmin && !lquery) info = -10;
      else if (*LIWORK < liwmin && !lquery) info = -12;
    }
  }
  *INFO = info;
  if (info != 0) { pxerbla(DESCA[CTXT_], "PDGECON", -info); return; }
  if (lquery) return;
  *RCOND = 0.0;
  if (n == 0) { *RCOND = 1.0; return; }
  if (*ANORM == 0.0) return;
  if (n == 1) { *RCOND = 1.0; return; }
  double* dA = nullptr;
  long long ldda = 0;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!ensure_device()) { *INFO = cuda_info(cudaErrorNoDevice); return; }
    ldda = round_ld(n);
    cudaError_t e = grow(&g_dev.dA, &g_dev.capA, (size_t)ldda * n);
    const long long lld = DESCA[LLD_];
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(g_dev.dA, ldda * sizeof(double), A + (ia - 1) + (long long)(ja - 1) * lld,
                            lld * sizeof(double), (size_t)n * sizeof(double), n,
                            cudaMemcpyHostToDevice, g_dev.stream);
    if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
    dA = g_dev.dA;
  }
  *INFO = sl1x1_dgecon_dev(NORM[0], n, dA, ldda, *ANORM, RCOND, g_dev.stream);
}

int sl1x1_dgetri_dev(int n, double* dA, long long ldda, const int* dipiv, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (n < 0) return -1;
  if (ldda < (n > 1 ? n : 1)) return -3;
  if (n == 0) return 0;
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = grow(&g_dev.dipiv, &g_dev.capP, (size_t)n);
  if (e == cudaSuccess) e = ensure_solve_ws(n, n);
  if (e == cudaSuccess) e = grow(&g_dev.daux, &g_dev.capAux, (size_t)n * n + 8);
  if (e != cudaSuccess) return cuda_info(e);
  e = sl::ipiv_shift(dipiv, g_dev.dipiv, n, -1, s);
  if (e != cudaSuccess) return cuda_info(e);
  int info = 0;
  sl::LuWork w = make_work();
  e = sl::dgetri_device(n, dA, ldda, g_dev.dipiv, g_dev.daux, w,
                        reinterpret_cast<int*>(g_dev.daux + (size_t)n * n), &info, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? info : cuda_info(e);
}

// PDGETRI (SRC/pdgetri.f): validation and workspace query as the reference,
// inverse computed on the GPU from the LU factors and pivots of PDGETRF.
void pdgetri_(const int* N, double* A, const int* IA, const int* JA, const int* DESCA,
              const int* IPIV, double* WORK, const int* LWORK, int* IWORK, const int* LIWORK,
              int* INFO) {
  int nprow, npcol, myrow, mycol;
  gridinfo(DESCA[CTXT_], &nprow, &npcol, &myrow, &mycol);
  int info = 0;
  const int n = *N, ia = *IA, ja = *JA;
  bool lquery = false;
  if (nprow == -1) {
    info = -(500 + FCTXT);
  } else {
    chk1mat(n, 1, n, 1, ia, ja, DESCA, 5, &info);
    if (info == 0) {
      const int iroff = (ia - 1) % DESCA[MB_], icoff = (ja - 1) % DESCA[NB_];
      const int np = numroc(n + iroff, DESCA[MB_], 0, 0, 1);
      const int lwmin = np * DESCA[NB_];
      const int nq = numroc(DESCA[N_], DESCA[NB_], 0, 0, 1);
      const int liwmin = nq + DESCA[NB_];  // NPROW == NPCOL on a 1x1 grid
      WORK[0] = (double)lwmin;
      IWORK[0] = liwmin;
      lquery = (*LWORK == -1 || *LIWORK == -1);
      if (iroff != icoff || iroff != 0) info = -4;
      else if (DESCA[MB_] != DESCA[NB_]) info = -(500 + FNB);
      else if (*LWORK < lwmin && !lquery) info = -8;
      else if (*LIWORK < liwmin && !lquery) info = -10;
    }
  }
  *INFO = info;
  if (info != 0) { pxerbla(DESCA[CTXT_], "PDGETRI", -info); return; }
  if (lquery || n == 0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!ensure_device()) { *INFO = cuda_info(cudaErrorNoDevice); return; }
  const long long lld = DESCA[LLD_];
  const long long ldda = round_ld(n);
  cudaStream_t s = g_dev.stream;
  cudaError_t e = grow(&g_dev.dA, &g_dev.capA, (size_t)ldda * n);
  if (e == cudaSuccess) e = grow(&g_dev.dipiv, &g_dev.capP, (size_t)n);
  if (e == cudaSuccess) e = ensure_solve_ws(n, n);
  if (e == cudaSuccess) e = grow(&g_dev.daux, &g_dev.capAux, (size_t)n * n + 8);
  if (e != cudaSuccess) { *INFO = cuda_info(e); return; }
  double* hA = A + (ia - 1) + (long long)(ja - 1) * lld;
  std::vector<int> hp((size_t)n);
  for (int k = 0; k < n; ++k) hp[k] = IPIV[ia - 1 + k] - ia;
  e = cudaMemcpy2DAsync(g_dev.dA, ldda * sizeof(double), hA, lld * sizeof(double),
                        (size_t)n * sizeof(double), n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(g_dev.dipiv, hp.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s);
  int dinfo = 0;
  sl::LuWork w = make_work();
  if (e == cudaSuccess)
    e = sl::dgetri_device(n, g_dev.dA, ldda, g_dev.dipiv, g_dev.daux, w,
                          reinterpret_cast<int*>(g_dev.daux + (size_t)n * n), &dinfo, s);
  if (e == cudaSuccess && dinfo == 0)
    e = cudaMemcpy2DAsync(hA, lld * sizeof(double), g_dev.dA, ldda * sizeof(double),
                          (size_t)n * sizeof(double), n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  *INFO = (e == cudaSuccess) ? dinfo : cuda_info(e);
}

void sl1x1_finalize(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  release_all();
}

void sl1x1_set_lookahead(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_lookahead = (on != 0);
}

void sl1x1_set_split_step(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_split_step = (on != 0);
}

int sl1x1_debug_fail_alloc(int k) {
  std::lock_guard<std::mutex> lk(g_mu);
  const int prev = g_fail_alloc_in;
  g_fail_alloc_in = k < 0 ? -1 : k;
  return prev;
}

void sl1x1_set_copy_chunks(int chunks) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_copy_chunks = chunks < 1 ? 1 : (chunks > sl::kMaxColChunks ? sl::kMaxColChunks : chunks);
}

void sl1x1_set_panel_ib(int subpanels) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::set_panel_ib(subpanels);
}

void sl1x1_set_panel_ctas(int ctas) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::set_panel_ctas(ctas);
}

void sl1x1_set_panel_rows(int rows) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::set_panel_min_rows(rows);
}

void sl1x1_set_lowp_stages(int stages) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::lowp_set_stages(stages);
}

void sl1x1_set_f64_update(int mode) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::f64_update_set(mode);
}

void sl1x1_set_ozgemm_tiles(int tiles_per_cta) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::oz_set_tiles_per_cta(tiles_per_cta);
}

int sl1x1_get_f64_update(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return sl::f64_update_get();
}

int sl1x1_ozgemm_dev(int m, int n, int k, double alpha, const double* dA, long long ldda,
                     const double* dB, long long lddb, double* dC, long long lddc, void* stream) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (m < 0) return -1;
  if (n < 0) return -2;
  if (k < 0) return -3;
  if (ldda < (m > 1 ? m : 1)) return -6;
  if (lddb < (k > 1 ? k : 1)) return -8;
  if (lddc < (m > 1 ? m : 1)) return -10;
  if (m == 0 || n == 0 || k == 0) return 0;
  if (!ensure_device()) return cuda_info(cudaErrorNoDevice);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t need = sl::oz_scratch_bytes(m, n, k);
  if (need > g_dev.capOz || !g_dev.doz) {
    cudaError_t e = grow_oz(&g_dev.doz, &g_dev.capOz, need);
    if (e != cudaSuccess) return cuda_info(e);
  }
  sl::OzScratch sc;
  sc.ptr = g_dev.doz;
  sc.bytes = g_dev.capOz;
  cudaError_t e = cudaMemsetAsync(g_dev.dsmall + 2, 0, sizeof(int), s);
  if (e == cudaSuccess) e = sl::oz_dgemm(sc, m, n, k, alpha, dA, ldda, dB, lddb, dC, lddc, g_dev.dsmall + 2, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_info(e);
  int st = 0;
  e = cudaMemcpy(&st, g_dev.dsmall + 2, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_info(e);
  return st ? -20000 - st : 0;
}

void sl1x1_set_update_reserve(int min_sms, int max_sms) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::set_update_reserve(min_sms, max_sms);
}

void sl1x1_set_inpanel_cap(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::set_inpanel_cap(on);
}

void sl1x1_set_update_share(double flops_per_sm) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::set_update_share(flops_per_sm);
}

void sl1x1_debug_set_spin_limit(long long polls) {
  std::lock_guard<std::mutex> lk(g_mu);
  sl::set_spin_limit(polls);
}

void sl1x1_set_ir_cost_ratio(double ratio) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_ir_cost_ratio = ratio > 0.0 ? ratio : 0.0;
}

long long sl1x1_ozgemm_fp64_routes(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!ensure_device()) return -1;
  return sl::oz_fp64_routes();
}

void sl1x1_set_default_nb(int nb) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (nb > 0) g_default_nb = nb;
}

int sl1x1_device_ok(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  return ensure_device() ? 1 : 0;
}

const char* sl1x1_version(void) { return "sl1x1-gb300 0.1 (sm_103a)"; }

void sl1x1_prof_enable(int on) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!ensure_device()) return;
  sl::prof_enable(on != 0);
}

int sl1x1_prof_read(int phase, long long* launches, double* ms, double* flops, double* bytes) {
  std::lock_guard<std::mutex> lk(g_mu);
  return sl::prof_read(phase, launches, ms, flops, bytes) ? 0 : -1;
}

long long sl1x1_launch_count(void) { return sl::launch_count(); }

double sl1x1_dmma_peak_tflops(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!ensure_device()) return 0.0;
  return sl::dmma_peak_tflops(g_dev.stream);
}

}  // extern "C"
