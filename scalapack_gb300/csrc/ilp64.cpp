// ILP64 Fortran ABI (include/sl1x1_ilp64.h): the reference's entry points for
// callers built with 8-byte INTEGERs (the "Int=long" build, README:145-154),
// forwarded to the 32-bit entry points of libsl1x1gpu.so, which this library
// loads privately (RTLD_LOCAL) from its own directory. Every INTEGER is
// narrowed on the way in and widened on the way out; a value outside the
// 32-bit range is an illegal argument: INFO = -(position), or -(100 *
// position + entry) for a descriptor entry (the reference's encoding).
#include <dlfcn.h>

#include <climits>
#include <string>
#include <vector>

#include "../../include/sl1x1_ilp64.h"

namespace {

using i64 = sl_int64;
constexpr i64 kNoLibrary = -19999;  // libsl1x1gpu.so not found beside this library

void* main_lib() {
  static void* h = [] {
    Dl_info info;
    std::string dir = ".";
    if (dladdr(reinterpret_cast<void*>(&main_lib), &info) && info.dli_fname) {
      dir = info.dli_fname;
      const size_t p = dir.rfind('/');
      dir = (p == std::string::npos) ? std::string(".") : dir.substr(0, p);
    }
    return dlopen((dir + "/libsl1x1gpu.so").c_str(), RTLD_NOW | RTLD_LOCAL);
  }();
  return h;
}

template <class F>
F entry(const char* name) {
  void* h = main_lib();
  return h ? reinterpret_cast<F>(dlsym(h, name)) : nullptr;
}

bool fits(i64 v) { return v >= INT_MIN && v <= INT_MAX; }

// Narrowed scalars and descriptors; `bad` keeps the first failure's INFO.
struct Args {
  i64 bad = 0;
  int s(const i64* v, int pos) {
    if (bad == 0 && !fits(*v)) bad = -pos;
    return (int)*v;
  }
  void d(const i64* D, int pos, int* out) {
    for (int e = 0; e < 9; ++e) {
      if (bad == 0 && !fits(D[e])) bad = -(100 * pos + e + 1);
      out[e] = (int)D[e];
    }
  }
};

// A 32-bit IPIV buffer for the entries IPIV(IA..IA+cnt-1) of a caller's
// 64-bit array (index IA-1+k): the 1x1 routines read and write only those.
// `ok` is false when the buffer would exceed 2^28 entries (an IA or N no
// matrix in device memory can have).
struct Piv {
  std::vector<int> v;
  int ia, cnt;
  bool ok;
  Piv(int ia_, int cnt_) : ia(ia_ > 0 ? ia_ : 1), cnt(cnt_ > 0 ? cnt_ : 0) {
    const long long len = (long long)(ia - 1) + cnt + 1;
    ok = len <= (1LL << 28);
    v.assign(ok ? (size_t)len : 1, 0);
  }
  bool load(const i64* src) {
    for (int k = 0; k < cnt; ++k) {
      const i64 x = src[ia - 1 + k];
      if (!fits(x)) return false;
      v[(size_t)(ia - 1 + k)] = (int)x;
    }
    return true;
  }
  void store(i64* dst) const {
    for (int k = 0; k < cnt; ++k) dst[ia - 1 + k] = v[(size_t)(ia - 1 + k)];
  }
};

// A 32-bit IWORK of at most 2^26 entries (the routines here need N + a few);
// its first entry starts as the caller's IWORK(1) and goes back to it.
struct IWork {
  std::vector<int> v;
  int len;
  IWork(int liwork, const i64* caller) {
    len = liwork < 1 ? liwork : (liwork > (1 << 26) ? (1 << 26) : liwork);
    v.assign((size_t)(len > 1 ? len : 1), 0);
    v[0] = fits(caller[0]) ? (int)caller[0] : 0;
  }
};

}  // namespace

extern "C" {

void pdgetrf_(const i64* M, const i64* N, double* A, const i64* IA, const i64* JA,
              const i64* DESCA, i64* IPIV, i64* INFO) {
  using F = void (*)(const int*, const int*, double*, const int*, const int*, const int*, int*, int*);
  static F f = entry<F>("pdgetrf_");
  if (!f) { *INFO = kNoLibrary; return; }
  Args a;
  int da[9];
  int m = a.s(M, 1), n = a.s(N, 2), ia = a.s(IA, 4), ja = a.s(JA, 5);
  a.d(DESCA, 6, da);
  if (a.bad) { *INFO = a.bad; return; }
  Piv p(ia, (m < n ? m : n));
  if (!p.ok) { *INFO = -4; return; }
  int info = 0;
  f(&m, &n, A, &ia, &ja, da, p.v.data(), &info);
  if (info >= 0 || info <= -10000) p.store(IPIV);
  *INFO = info;
}

void pdgetrs_(const char* TRANS, const i64* N, const i64* NRHS, const double* A, const i64* IA,
              const i64* JA, const i64* DESCA, const i64* IPIV, double* B, const i64* IB,
              const i64* JB, const i64* DESCB, i64* INFO, size_t TRANS_len) {
  using F = void (*)(const char*, const int*, const int*, const double*, const int*, const int*,
                     const int*, const int*, double*, const int*, const int*, const int*, int*,
                     size_t);
  static F f = entry<F>("pdgetrs_");
  if (!f) { *INFO = kNoLibrary; return; }
  Args a;
  int da[9], db[9];
  int n = a.s(N, 2), nrhs = a.s(NRHS, 3), ia = a.s(IA, 5), ja = a.s(JA, 6);
  a.d(DESCA, 7, da);
  int ib = a.s(IB, 10), jb = a.s(JB, 11);
  a.d(DESCB, 12, db);
  if (a.bad) { *INFO = a.bad; return; }
  Piv p(ia, n);
  if (!p.ok) { *INFO = -5; return; }
  if (n > 0 && ia >= 1 && !p.load(IPIV)) { *INFO = -8; return; }
  int info = 0;
  f(TRANS, &n, &nrhs, A, &ia, &ja, da, p.v.data(), B, &ib, &jb, db, &info, TRANS_len);
  *INFO = info;
}

void pdgesv_(const i64* N, const i64* NRHS, double* A, const i64* IA, const i64* JA,
             const i64* DESCA, i64* IPIV, double* B, const i64* IB, const i64* JB,
             const i64* DESCB, i64* INFO) {
  using F = void (*)(const int*, const int*, double*, const int*, const int*, const int*, int*,
                     double*, const int*, const int*, const int*, int*);
  static F f = entry<F>("pdgesv_");
  if (!f) { *INFO = kNoLibrary; return; }
  Args a;
  int da[9], db[9];
  int n = a.s(N, 1), nrhs = a.s(NRHS, 2), ia = a.s(IA, 4), ja = a.s(JA, 5);
  a.d(DESCA, 6, da);
  int ib = a.s(IB, 9), jb = a.s(JB, 10);
  a.d(DESCB, 11, db);
  if (a.bad) { *INFO = a.bad; return; }
  Piv p(ia, n);
  if (!p.ok) { *INFO = -4; return; }
  int info = 0;
  f(&n, &nrhs, A, &ia, &ja, da, p.v.data(), B, &ib, &jb, db, &info);
  if (info >= 0 || info <= -10000) p.store(IPIV);
  *INFO = info;
}

double pdlange_(const char* NORM, const i64* M, const i64* N, const double* A, const i64* IA,
                const i64* JA, const i64* DESCA, double* WORK, size_t NORM_len) {
  using F = double (*)(const char*, const int*, const int*, const double*, const int*, const int*,
                       const int*, double*, size_t);
  static F f = entry<F>("pdlange_");
  if (!f) return 0.0;
  Args a;
  int da[9];
  int m = a.s(M, 2), n = a.s(N, 3), ia = a.s(IA, 5), ja = a.s(JA, 6);
  a.d(DESCA, 7, da);
  if (a.bad) return 0.0;
  return f(NORM, &m, &n, A, &ia, &ja, da, WORK, NORM_len);
}

void pdgecon_(const char* NORM, const i64* N, const double* A, const i64* IA, const i64* JA,
              const i64* DESCA, const double* ANORM, double* RCOND, double* WORK,
              const i64* LWORK, i64* IWORK, const i64* LIWORK, i64* INFO, size_t NORM_len) {
  using F = void (*)(const char*, const int*, const double*, const int*, const int*, const int*,
                     const double*, double*, double*, const int*, int*, const int*, int*, size_t);
  static F f = entry<F>("pdgecon_");
  if (!f) { *INFO = kNoLibrary; return; }
  Args a;
  int da[9];
  int n = a.s(N, 2), ia = a.s(IA, 4), ja = a.s(JA, 5);
  a.d(DESCA, 6, da);
  int lwork = a.s(LWORK, 10), liwork = a.s(LIWORK, 12);
  if (a.bad) { *INFO = a.bad; return; }
  IWork iw(liwork, IWORK);
  int info = 0;
  f(NORM, &n, A, &ia, &ja, da, ANORM, RCOND, WORK, &lwork, iw.v.data(), &iw.len, &info, NORM_len);
  IWORK[0] = iw.v[0];
  *INFO = info;
}

void pdgetri_(const i64* N, double* A, const i64* IA, const i64* JA, const i64* DESCA,
              const i64* IPIV, double* WORK, const i64* LWORK, i64* IWORK, const i64* LIWORK,
              i64* INFO) {
  using F = void (*)(const int*, double*, const int*, const int*, const int*, const int*, double*,
                     const int*, int*, const int*, int*);
  static F f = entry<F>("pdgetri_");
  if (!f) { *INFO = kNoLibrary; return; }
  Args a;
  int da[9];
  int n = a.s(N, 1), ia = a.s(IA, 3), ja = a.s(JA, 4);
  a.d(DESCA, 5, da);
  int lwork = a.s(LWORK, 8), liwork = a.s(LIWORK, 10);
  if (a.bad) { *INFO = a.bad; return; }
  Piv p(ia, n);
  if (!p.ok) { *INFO = -3; return; }
  const bool query = (lwork == -1 || liwork == -1);
  if (!query && n > 0 && ia >= 1 && !p.load(IPIV)) { *INFO = -6; return; }
  IWork iw(liwork, IWORK);
  int info = 0;
  f(&n, A, &ia, &ja, da, p.v.data(), WORK, &lwork, iw.v.data(), &iw.len, &info);
  IWORK[0] = iw.v[0];
  *INFO = info;
}

void pdgerfs_(const char* TRANS, const i64* N, const i64* NRHS, const double* A, const i64* IA,
              const i64* JA, const i64* DESCA, const double* AF, const i64* IAF, const i64* JAF,
              const i64* DESCAF, const i64* IPIV, const double* B, const i64* IB, const i64* JB,
              const i64* DESCB, double* X, const i64* IX, const i64* JX, const i64* DESCX,
              double* FERR, double* BERR, double* WORK, const i64* LWORK, i64* IWORK,
              const i64* LIWORK, i64* INFO, size_t TRANS_len) {
  using F = void (*)(const char*, const int*, const int*, const double*, const int*, const int*,
                     const int*, const double*, const int*, const int*, const int*, const int*,
                     const double*, const int*, const int*, const int*, double*, const int*,
                     const int*, const int*, double*, double*, double*, const int*, int*,
                     const int*, int*, size_t);
  static F f = entry<F>("pdgerfs_");
  if (!f) { *INFO = kNoLibrary; return; }
  Args a;
  int da[9], daf[9], db[9], dx[9];
  int n = a.s(N, 2), nrhs = a.s(NRHS, 3), ia = a.s(IA, 5), ja = a.s(JA, 6);
  a.d(DESCA, 7, da);
  int iaf = a.s(IAF, 9), jaf = a.s(JAF, 10);
  a.d(DESCAF, 11, daf);
  int ib = a.s(IB, 14), jb = a.s(JB, 15);
  a.d(DESCB, 16, db);
  int ix = a.s(IX, 18), jx = a.s(JX, 19);
  a.d(DESCX, 20, dx);
  int lwork = a.s(LWORK, 24), liwork = a.s(LIWORK, 26);
  if (a.bad) { *INFO = a.bad; return; }
  Piv p(iaf, n);
  if (!p.ok) { *INFO = -9; return; }
  const bool query = (lwork == -1 || liwork == -1);
  if (!query && n > 0 && iaf >= 1 && !p.load(IPIV)) { *INFO = -12; return; }
  IWork iw(liwork, IWORK);
  int info = 0;
  f(TRANS, &n, &nrhs, A, &ia, &ja, da, AF, &iaf, &jaf, daf, p.v.data(), B, &ib, &jb, db, X, &ix,
    &jx, dx, FERR, BERR, WORK, &lwork, iw.v.data(), &iw.len, &info, TRANS_len);
  IWORK[0] = iw.v[0];
  *INFO = info;
}

void pdgesvx_(const char* FACT, const char* TRANS, const i64* N, const i64* NRHS, double* A,
              const i64* IA, const i64* JA, const i64* DESCA, double* AF, const i64* IAF,
              const i64* JAF, const i64* DESCAF, i64* IPIV, char* EQUED, double* R, double* C,
              double* B, const i64* IB, const i64* JB, const i64* DESCB, double* X, const i64* IX,
              const i64* JX, const i64* DESCX, double* RCOND, double* FERR, double* BERR,
              double* WORK, const i64* LWORK, i64* IWORK, const i64* LIWORK, i64* INFO,
              size_t FACT_len, size_t TRANS_len, size_t EQUED_len) {
  using F = void (*)(const char*, const char*, const int*, const int*, double*, const int*,
                     const int*, const int*, double*, const int*, const int*, const int*, int*,
                     char*, double*, double*, double*, const int*, const int*, const int*, double*,
                     const int*, const int*, const int*, double*, double*, double*, double*,
                     const int*, int*, const int*, int*, size_t, size_t, size_t);
  static F f = entry<F>("pdgesvx_");
  if (!f) { *INFO = kNoLibrary; return; }
  Args a;
  int da[9], daf[9], db[9], dx[9];
  int n = a.s(N, 3), nrhs = a.s(NRHS, 4), ia = a.s(IA, 6), ja = a.s(JA, 7);
  a.d(DESCA, 8, da);
  int iaf = a.s(IAF, 10), jaf = a.s(JAF, 11);
  a.d(DESCAF, 12, daf);
  int ib = a.s(IB, 18), jb = a.s(JB, 19);
  a.d(DESCB, 20, db);
  int ix = a.s(IX, 22), jx = a.s(JX, 23);
  a.d(DESCX, 24, dx);
  int lwork = a.s(LWORK, 29), liwork = a.s(LIWORK, 31);
  if (a.bad) { *INFO = a.bad; return; }
  Piv p(iaf, n);
  if (!p.ok) { *INFO = -10; return; }
  const bool fact_f = (FACT[0] == 'F' || FACT[0] == 'f');
  const bool query = (lwork == -1 || liwork == -1);
  if (fact_f && !query && n > 0 && iaf >= 1 && !p.load(IPIV)) { *INFO = -13; return; }
  IWork iw(liwork, IWORK);
  int info = 0;
  f(FACT, TRANS, &n, &nrhs, A, &ia, &ja, da, AF, &iaf, &jaf, daf, p.v.data(), EQUED, R, C, B, &ib,
    &jb, db, X, &ix, &jx, dx, RCOND, FERR, BERR, WORK, &lwork, iw.v.data(), &iw.len, &info,
    FACT_len, TRANS_len, EQUED_len);
  if (!fact_f && !query && (info >= 0 || info <= -10000) && n > 0 && iaf >= 1) p.store(IPIV);
  IWORK[0] = iw.v[0];
  *INFO = info;
}

void pdgeequ_(const i64* M, const i64* N, const double* A, const i64* IA, const i64* JA,
              const i64* DESCA, double* R, double* C, double* ROWCND, double* COLCND,
              double* AMAX, i64* INFO) {
  using F = void (*)(const int*, const int*, const double*, const int*, const int*, const int*,
                     double*, double*, double*, double*, double*, int*);
  static F f = entry<F>("pdgeequ_");
  if (!f) { *INFO = kNoLibrary; return; }
  Args a;
  int da[9];
  int m = a.s(M, 1), n = a.s(N, 2), ia = a.s(IA, 4), ja = a.s(JA, 5);
  a.d(DESCA, 6, da);
  if (a.bad) { *INFO = a.bad; return; }
  int info = 0;
  f(&m, &n, A, &ia, &ja, da, R, C, ROWCND, COLCND, AMAX, &info);
  *INFO = info;
}

void pdlaqge_(const i64* M, const i64* N, double* A, const i64* IA, const i64* JA,
              const i64* DESCA, const double* R, const double* C, const double* ROWCND,
              const double* COLCND, const double* AMAX, char* EQUED, size_t EQUED_len) {
  using F = void (*)(const int*, const int*, double*, const int*, const int*, const int*,
                     const double*, const double*, const double*, const double*, const double*,
                     char*, size_t);
  static F f = entry<F>("pdlaqge_");
  if (!f) return;
  Args a;
  int da[9];
  int m = a.s(M, 1), n = a.s(N, 2), ia = a.s(IA, 4), ja = a.s(JA, 5);
  a.d(DESCA, 6, da);
  if (a.bad) return;
  f(&m, &n, A, &ia, &ja, da, R, C, ROWCND, COLCND, AMAX, EQUED, EQUED_len);
}

void pdgemr2d_(const i64* M, const i64* N, const double* A, const i64* IA, const i64* JA,
               const i64* DESCA, double* B, const i64* IB, const i64* JB, const i64* DESCB,
               const i64* ICTXT) {
  using F = void (*)(const int*, const int*, const double*, const int*, const int*, const int*,
                     double*, const int*, const int*, const int*, const int*);
  static F f = entry<F>("pdgemr2d_");
  if (!f) return;
  Args a;
  int da[9], db[9];
  int m = a.s(M, 1), n = a.s(N, 2), ia = a.s(IA, 4), ja = a.s(JA, 5);
  a.d(DESCA, 6, da);
  int ib = a.s(IB, 8), jb = a.s(JB, 9);
  a.d(DESCB, 10, db);
  int ctxt = a.s(ICTXT, 11);
  if (a.bad) return;
  f(&m, &n, A, &ia, &ja, da, B, &ib, &jb, db, &ctxt);
}

void descinit_(i64* DESC, const i64* M, const i64* N, const i64* MB, const i64* NB,
               const i64* IRSRC, const i64* ICSRC, const i64* ICTXT, const i64* LLD, i64* INFO) {
  using F = void (*)(int*, const int*, const int*, const int*, const int*, const int*, const int*,
                     const int*, const int*, int*);
  static F f = entry<F>("descinit_");
  if (!f) { *INFO = kNoLibrary; return; }
  Args a;
  int m = a.s(M, 2), n = a.s(N, 3), mb = a.s(MB, 4), nb = a.s(NB, 5), rs = a.s(IRSRC, 6),
      cs = a.s(ICSRC, 7), ctxt = a.s(ICTXT, 8), lld = a.s(LLD, 9);
  if (a.bad) { *INFO = a.bad; return; }
  int d[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int info = 0;
  f(d, &m, &n, &mb, &nb, &rs, &cs, &ctxt, &lld, &info);
  for (int e = 0; e < 9; ++e) DESC[e] = d[e];
  *INFO = info;
}

i64 numroc_(const i64* N, const i64* NB, const i64* IPROC, const i64* ISRCPROC, const i64* NPROCS) {
  // TOOLS/numroc.f:53-76, in 64-bit arithmetic
  const i64 n = *N, nb = *NB, nprocs = *NPROCS;
  const i64 mydist = (nprocs + *IPROC - *ISRCPROC) % nprocs;
  const i64 nblocks = n / nb;
  i64 r = (nblocks / nprocs) * nb;
  const i64 extra = nblocks % nprocs;
  if (mydist < extra) r += nb;
  else if (mydist == extra) r += n % nb;
  return r;
}

void blacs_pinfo_(i64* MYPNUM, i64* NPROCS) {
  using F = void (*)(int*, int*);
  static F f = entry<F>("blacs_pinfo_");
  int me = 0, np = 0;
  if (f) f(&me, &np);
  *MYPNUM = me;
  *NPROCS = np;
}

void blacs_get_(const i64* ICTXT, const i64* WHAT, i64* VAL) {
  using F = void (*)(const int*, const int*, int*);
  static F f = entry<F>("blacs_get_");
  int c = fits(*ICTXT) ? (int)*ICTXT : -1, w = fits(*WHAT) ? (int)*WHAT : -1, v = 0;
  if (f) f(&c, &w, &v);
  *VAL = v;
}

void blacs_gridinit_(i64* ICTXT, const char* ORDER, const i64* NPROW, const i64* NPCOL,
                     size_t ORDER_len) {
  using F = void (*)(int*, const char*, const int*, const int*, size_t);
  static F f = entry<F>("blacs_gridinit_");
  int c = fits(*ICTXT) ? (int)*ICTXT : 0;
  const int pr = fits(*NPROW) ? (int)*NPROW : -1, pc = fits(*NPCOL) ? (int)*NPCOL : -1;
  if (f) f(&c, ORDER, &pr, &pc, ORDER_len);
  *ICTXT = c;
}

void blacs_gridinfo_(const i64* ICTXT, i64* NPROW, i64* NPCOL, i64* MYROW, i64* MYCOL) {
  using F = void (*)(const int*, int*, int*, int*, int*);
  static F f = entry<F>("blacs_gridinfo_");
  const int c = fits(*ICTXT) ? (int)*ICTXT : -1;
  int pr = -1, pc = -1, r = -1, col = -1;
  if (f) f(&c, &pr, &pc, &r, &col);
  *NPROW = pr;
  *NPCOL = pc;
  *MYROW = r;
  *MYCOL = col;
}

void blacs_gridexit_(const i64* ICTXT) {
  using F = void (*)(const int*);
  static F f = entry<F>("blacs_gridexit_");
  const int c = fits(*ICTXT) ? (int)*ICTXT : -1;
  if (f) f(&c);
}

void blacs_exit_(const i64* CONTINUE) {
  using F = void (*)(const int*);
  static F f = entry<F>("blacs_exit_");
  const int c = fits(*CONTINUE) ? (int)*CONTINUE : 0;
  if (f) f(&c);
}

}  // extern "C"
