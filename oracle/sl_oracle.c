/*
 * sl_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of ScaLAPACK 2.2.3's dense LU path on a 1x1 BLACS grid
 * (PDGETRF / PDGETF2 / PDLASWP / PDTRSM / PDGEMM / PDGETRS / PDLAPIV), of the
 * expert driver around it (PDGEEQU / PDLAQGE / PDLANGE / PDGECON / PDLACON /
 * PDGERFS / PDGESVX) and of the LU tester's generator and residual checks.  It is the checker that the GPU
 * library is compared against; it is never linked into, called by, or used as
 * a fallback for the product library.  Only the test suite, the smoke check
 * and the CPU-baseline leg of the benchmark load it.
 *
 * Parity anchor: the reference cannot be compiled in this environment (it is
 * Fortran 77 over MPI and no Fortran compiler or MPI is installed), so this
 * restatement is pinned against (a) the EXAMPLE/DSCAEX{MAT,RHS}.dat known-answer
 * system, (b) LAPACK DGETRF/DGETRS from the host BLAS (same pivoting rule, IPIV
 * compared entry by entry) and (c) the LU.dat tester sizes with the tester's
 * scaled-residual thresholds.
 *
 * Host BLAS: the local BLAS the reference calls (dgemm, dtrsm, dger, dscal,
 * dswap, idamax) are bound at run time by orc_load_blas() from a shared
 * library (scipy's bundled OpenBLAS, exported with a "scipy_" prefix).  When no
 * library is loaded, plain C loops with reference-BLAS semantics are used, so
 * the oracle always runs (slowly) for small cases.
 *
 * All index arguments are 1-based Fortran-style where the reference uses them.
 */
#include <dlfcn.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int blasint;

/* ------------------------------------------------------------------------- */
/* BLAS binding                                                               */
/* ------------------------------------------------------------------------- */
typedef void (*dgemm_t)(const char*, const char*, const blasint*, const blasint*, const blasint*,
                        const double*, const double*, const blasint*, const double*, const blasint*,
                        const double*, double*, const blasint*, size_t, size_t);
typedef void (*dtrsm_t)(const char*, const char*, const char*, const char*, const blasint*,
                        const blasint*, const double*, const double*, const blasint*, double*,
                        const blasint*, size_t, size_t, size_t, size_t);
typedef void (*dger_t)(const blasint*, const blasint*, const double*, const double*, const blasint*,
                       const double*, const blasint*, double*, const blasint*);
typedef void (*dscal_t)(const blasint*, const double*, double*, const blasint*);
typedef void (*dswap_t)(const blasint*, double*, const blasint*, double*, const blasint*);
typedef blasint (*idamax_t)(const blasint*, const double*, const blasint*);
typedef void (*dgetrf_t)(const blasint*, const blasint*, double*, const blasint*, blasint*, blasint*);
typedef void (*dgetrs_t)(const char*, const blasint*, const blasint*, const double*, const blasint*,
                         const blasint*, double*, const blasint*, blasint*, size_t);
typedef void (*setthr_t)(int);

static dgemm_t p_dgemm;
static dtrsm_t p_dtrsm;
static dger_t p_dger;
static dscal_t p_dscal;
static dswap_t p_dswap;
static idamax_t p_idamax;
static dgetrf_t p_dgetrf;
static dgetrs_t p_dgetrs;
static setthr_t p_setthr;
static void* blas_handle;

/* Plain-loop fallbacks with reference-BLAS semantics (column-major). */
static blasint c_idamax(const blasint* n, const double* x, const blasint* incx) {
  /* Reference BLAS IDAMAX: first index of max |x|, strict '>' so ties keep the
   * first one and a NaN never replaces the running maximum. */
  if (*n < 1 || *incx <= 0) return 0;
  blasint best = 1;
  double dmax = fabs(x[0]);
  for (blasint i = 1; i < *n; ++i) {
    double v = fabs(x[(size_t)i * *incx]);
    if (v > dmax) { best = i + 1; dmax = v; }
  }
  return best;
}
static void c_dswap(const blasint* n, double* x, const blasint* incx, double* y, const blasint* incy) {
  for (blasint i = 0; i < *n; ++i) {
    double t = x[(size_t)i * *incx];
    x[(size_t)i * *incx] = y[(size_t)i * *incy];
    y[(size_t)i * *incy] = t;
  }
}
static void c_dscal(const blasint* n, const double* a, double* x, const blasint* incx) {
  for (blasint i = 0; i < *n; ++i) x[(size_t)i * *incx] *= *a;
}
static void c_dger(const blasint* m, const blasint* n, const double* alpha, const double* x,
                   const blasint* incx, const double* y, const blasint* incy, double* a,
                   const blasint* lda) {
  for (blasint j = 0; j < *n; ++j) {
    double t = *alpha * y[(size_t)j * *incy];
    if (t == 0.0) continue;
    for (blasint i = 0; i < *m; ++i) a[i + (size_t)j * *lda] += x[(size_t)i * *incx] * t;
  }
}
static void c_dgemm(const char* ta, const char* tb, const blasint* m, const blasint* n,
                    const blasint* k, const double* alpha, const double* a, const blasint* lda,
                    const double* b, const blasint* ldb, const double* beta, double* c,
                    const blasint* ldc, size_t l1, size_t l2) {
  (void)l1; (void)l2;
  int nta = (ta[0] == 'N' || ta[0] == 'n'), ntb = (tb[0] == 'N' || tb[0] == 'n');
  for (blasint j = 0; j < *n; ++j)
    for (blasint i = 0; i < *m; ++i) {
      double s = 0.0;
      for (blasint p = 0; p < *k; ++p) {
        double av = nta ? a[i + (size_t)p * *lda] : a[p + (size_t)i * *lda];
        double bv = ntb ? b[p + (size_t)j * *ldb] : b[j + (size_t)p * *ldb];
        s += av * bv;
      }
      double* cij = &c[i + (size_t)j * *ldc];
      *cij = (*beta == 0.0 ? 0.0 : *beta * *cij) + *alpha * s;
    }
}
/* Left-side triangular solve op(A)*X = alpha*B (the only side the LU path uses). */
static void c_dtrsm(const char* side, const char* uplo, const char* trans, const char* diag,
                    const blasint* m, const blasint* n, const double* alpha, const double* a,
                    const blasint* lda, double* b, const blasint* ldb, size_t l1, size_t l2,
                    size_t l3, size_t l4) {
  (void)side; (void)l1; (void)l2; (void)l3; (void)l4;
  int upper = (uplo[0] == 'U' || uplo[0] == 'u');
  int notr = (trans[0] == 'N' || trans[0] == 'n');
  int unit = (diag[0] == 'U' || diag[0] == 'u');
  blasint M = *m, LDA = *lda, LDB = *ldb;
#define AA(i, j) a[(i) + (size_t)(j) * LDA]
  for (blasint j = 0; j < *n; ++j) {
    double* x = b + (size_t)j * LDB;
    for (blasint i = 0; i < M; ++i) x[i] *= *alpha;
    /* Effective lower (forward) when (lower, N) or (upper, T). */
    int forward = (upper != notr);
    if (forward) {
      for (blasint i = 0; i < M; ++i) {
        double s = x[i];
        for (blasint p = 0; p < i; ++p) s -= (notr ? AA(i, p) : AA(p, i)) * x[p];
        x[i] = unit ? s : s / AA(i, i);
      }
    } else {
      for (blasint i = M - 1; i >= 0; --i) {
        double s = x[i];
        for (blasint p = i + 1; p < M; ++p) s -= (notr ? AA(i, p) : AA(p, i)) * x[p];
        x[i] = unit ? s : s / AA(i, i);
      }
    }
  }
#undef AA
}

static void bind_fallbacks(void) {
  p_dgemm = c_dgemm; p_dtrsm = c_dtrsm; p_dger = c_dger; p_dscal = c_dscal;
  p_dswap = c_dswap; p_idamax = c_idamax; p_dgetrf = NULL; p_dgetrs = NULL; p_setthr = NULL;
}

static void* sym(const char* prefix, const char* name) {
  char buf[256];
  snprintf(buf, sizeof buf, "%s%s", prefix, name);
  return dlsym(blas_handle, buf);
}

/* Bind the host BLAS from a shared library. Returns 0 on success, -1 if the
 * library cannot be opened or lacks a symbol (fallbacks stay bound). */
int orc_load_blas(const char* path, const char* prefix) {
  bind_fallbacks();
  if (!path || !path[0]) return -1;
  blas_handle = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!blas_handle) return -1;
  dgemm_t g = (dgemm_t)sym(prefix, "dgemm_");
  dtrsm_t t = (dtrsm_t)sym(prefix, "dtrsm_");
  dger_t r = (dger_t)sym(prefix, "dger_");
  dscal_t s = (dscal_t)sym(prefix, "dscal_");
  dswap_t w = (dswap_t)sym(prefix, "dswap_");
  idamax_t x = (idamax_t)sym(prefix, "idamax_");
  if (!g || !t || !r || !s || !w || !x) return -1;
  p_dgemm = g; p_dtrsm = t; p_dger = r; p_dscal = s; p_dswap = w; p_idamax = x;
  p_dgetrf = (dgetrf_t)sym(prefix, "dgetrf_");
  p_dgetrs = (dgetrs_t)sym(prefix, "dgetrs_");
  p_setthr = (setthr_t)sym(prefix, "openblas_set_num_threads");
  return 0;
}

/* Use the plain-loop BLAS again (tests use it to pin OpenBLAS against loops). */
void orc_use_fallback_blas(void) { bind_fallbacks(); }

int orc_blas_loaded(void) { return p_dgemm != NULL && p_dgemm != c_dgemm; }

void orc_set_threads(int n) { if (p_setthr) p_setthr(n); }

/* ------------------------------------------------------------------------- */
/* PDMATGEN generator (TESTING/traditional/LIN/pdmatgen.f, pmatgeninc.f)     */
/* ------------------------------------------------------------------------- */
/* The tester's LCG: x <- (1103515245*x + 12345) mod 2^31, the multiplier kept
 * as 16-bit halves MULT0=20077, MULT1=16838 and the increment IADD0=12345
 * (pdmatgen.f:116-118).  PDRAND returns x/2^31 and then advances
 * (pmatgeninc.f, PDRAND).  On a 1x1 grid the jump-ahead bookkeeping of
 * PDMATGEN reduces to: entry (i,j) of an M-row matrix (0-based) uses the state
 * advanced i + j*M steps from the first state a*seed + c. */
#define LCG_A 1103515245ULL
#define LCG_C 12345ULL
#define LCG_MASK 0x7fffffffULL

/* Affine map x -> A*x + C (mod 2^31) raised to the n-th power. */
static void lcg_jump(uint64_t n, uint64_t* An, uint64_t* Cn) {
  uint64_t ra = 1, rc = 0;          /* result map */
  uint64_t ba = LCG_A, bc = LCG_C;  /* base map */
  while (n) {
    if (n & 1) { /* result = base o result */
      rc = (ba * rc + bc) & LCG_MASK;
      ra = (ba * ra) & LCG_MASK;
    }
    /* base = base o base */
    bc = (ba * bc + bc) & LCG_MASK;
    ba = (ba * ba) & LCG_MASK;
    n >>= 1;
  }
  *An = ra; *Cn = rc;
}

/* State of the generator after `steps` draws for seed ISEED. */
uint32_t orc_lcg_state(int seed, uint64_t steps) {
  uint64_t x0 = ((uint64_t)(uint32_t)seed * LCG_A + LCG_C) & LCG_MASK;
  uint64_t An, Cn;
  lcg_jump(steps, &An, &Cn);
  return (uint32_t)((An * x0 + Cn) & LCG_MASK);
}

/*
 * Fill out(r,c) (leading dimension ldo) with entries (i0+r, j0+c) of the
 * M x N matrix PDMATGEN generates on a 1x1 grid with AFORM='N' and seed ISEED.
 *   kind 0: the tester's values 1 - 2*PDRAND, uniform on (-1,1]
 *           (pdmatgen.f, the general branch: A(IK,JK) = ONE - TWO*PDRAND(0)).
 *   kind 1: 0.5 - PDRAND, uniform on (-0.5,0.5] (the benchmark inputs).
 * diag != 0 applies DIAG='D': A(i,i) = |A(i,i)| + max(M,N) (pdmatgen.f, the
 * DIAG branch at the end).
 */
void orc_matgen(int M, int N, int seed, int kind, int diag, int i0, int j0, int nrows, int ncols,
                double* out, int ldo) {
  const double inv = 1.0 / 2147483648.0;
  int maxmn = M > N ? M : N;
  for (int c = 0; c < ncols; ++c) {
    int j = j0 + c;
    uint64_t x = orc_lcg_state(seed, (uint64_t)j * (uint64_t)M + (uint64_t)i0);
    for (int r = 0; r < nrows; ++r) {
      int i = i0 + r;
      double u = (double)x * inv;
      double v = kind == 0 ? 1.0 - 2.0 * u : 0.5 - u;
      if (diag && i == j) v = fabs(v) + (double)maxmn;
      out[r + (size_t)c * ldo] = v;
      x = (uint32_t)((LCG_A * x + LCG_C) & LCG_MASK);
    }
  }
}

/* ------------------------------------------------------------------------- */
/* Near-tie recorder and forced-pivot replay                                  */
/* ------------------------------------------------------------------------- */
/* For each factored column (0-based, relative to the submatrix) the panel
 * records the largest and second largest |candidate|.  When `force` is set,
 * the pivot of column k is taken from force[k] (1-based global row) instead of
 * IDAMAX, so that a comparison can continue past a logged near-tie. */
static double* g_top1;
static double* g_top2;
static const int* g_force;
static int g_ncols_rec;

void orc_set_recorder(double* top1, double* top2, int ncols, const int* force) {
  g_top1 = top1; g_top2 = top2; g_ncols_rec = ncols; g_force = force;
}

/* ------------------------------------------------------------------------- */
/* The 1x1 LU path                                                            */
/* ------------------------------------------------------------------------- */
#define A_(i, j) (A + ((size_t)(i) - 1) + ((size_t)(j) - 1) * (size_t)lda) /* 1-based */
static const double ONE = 1.0, MONE = -1.0;
static const blasint IONE = 1;

/* PDGETF2 on a 1x1 grid (SRC/pdgetf2.f:206-237). Factors the m x n panel
 * starting at global (ia, ja); IPIV is indexed by global row (IPIV(IA+J-JA)).
 * Returns INFO (first zero pivot, relative 1-based, or 0). */
static int pdgetf2_1x1(int m, int n, double* A, int lda, int ia, int ja, int* ipiv, int col0) {
  int info = 0;
  if (m == 0 || n == 0) return 0;
  int mn = m < n ? m : n;
  for (int j = ja; j <= ja + mn - 1; ++j) {
    int i = ia + j - ja;
    blasint len = m - j + ja;
    /* PDAMAX (PBLAS/SRC/pdamax_.c:414-486): first max |x| via IDAMAX, AMAX is
     * the signed entry; when AMAX is zero INDX is the first row. */
    blasint rel = p_idamax(&len, A_(i, j), &IONE);
    double gmax = *A_(i + rel - 1, j);
    int indx = (gmax == 0.0) ? i : i + rel - 1;
    int kcol = col0 + (j - ja);
    if (g_top1 && kcol < g_ncols_rec) {
      double t1 = -1.0, t2 = -1.0;
      for (blasint r = 0; r < len; ++r) {
        double v = fabs(*A_(i + r, j));
        if (v > t1) { t2 = t1; t1 = v; } else if (v > t2) { t2 = v; }
      }
      g_top1[kcol] = t1; g_top2[kcol] = t2;
    }
    if (g_force && kcol < g_ncols_rec && g_force[kcol] > 0) {
      indx = g_force[kcol];
      gmax = *A_(indx, j);
    }
    ipiv[i - 1] = indx;
    if (gmax != 0.0) {
      /* PDSWAP over the N panel columns (pdgetf2.f:218-219). */
      if (indx != i) {
        blasint nn = n;
        blasint ld = lda;
        p_dswap(&nn, A_(i, ja), &ld, A_(indx, ja), &ld);
      }
      /* PDSCAL by ONE/GMAX (pdgetf2.f:224-225): reciprocal, then multiply. */
      if (j - ja + 1 < m) {
        blasint cnt = m - j + ja - 1;
        double r = ONE / gmax;
        p_dscal(&cnt, &r, A_(i + 1, j), &IONE);
      }
    } else if (info == 0) {
      info = j - ja + 1;
    }
    /* PDGER rank-1 update (pdgetf2.f:233-235). */
    if (j - ja + 1 < mn) {
      blasint mm = m - j + ja - 1, nn = n - j + ja - 1, ld = lda;
      p_dger(&mm, &nn, &MONE, A_(i + 1, j), &IONE, A_(i, j + 1), &ld, A_(i + 1, j + 1), &ld);
    }
  }
  return info;
}

/* PDLASWP 'Forward','Rows' on a 1x1 grid (SRC/pdlaswp.f:163-172):
 * for I = K1..K2, swap rows I and IPIV(I) over n columns starting at ja. */
static void pdlaswp_fwd_1x1(int n, double* A, int lda, int ja, int k1, int k2, const int* ipiv) {
  if (n <= 0) return;
  blasint nn = n, ld = lda;
  for (int i = k1; i <= k2; ++i) {
    int ip = ipiv[i - 1];
    if (ip != i) p_dswap(&nn, A_(i, ja), &ld, A_(ip, ja), &ld);
  }
}

/* PDTRSM('L','L','N','U') on a 1x1 grid: PB_CptrsmAB's lower/no-transpose
 * loop (PBLAS/SRC/PTOOLS/PB_CptrsmAB.c:359-414) with kb = PILAENV = 32:
 * DTRSM on each 32-row diagonal block, DGEMM update of the rows below. */
static void trsm_lower_unit(int m, int n, const double* L, int ldl, double* B, int ldb) {
  const int kb = 32;
  for (int k = 0; k < m; k += kb) {
    blasint kbb = (m - k) < kb ? (m - k) : kb;
    blasint nn = n, l1 = ldl, l2 = ldb;
    p_dtrsm("L", "L", "N", "U", &kbb, &nn, &ONE, L + k + (size_t)k * ldl, &l1,
            B + k, &l2, 1, 1, 1, 1);
    blasint rest = m - k - kbb;
    if (rest > 0)
      p_dgemm("N", "N", &rest, &nn, &kbb, &MONE, L + (k + kbb) + (size_t)k * ldl, &l1, B + k, &l2,
              &ONE, B + k + kbb, &l2, 1, 1);
  }
}

/* PDTRSM('L','U','N','N'): PB_CptrsmAB's upper/no-transpose loop
 * (PB_CptrsmAB.c:309-357): blocks from the bottom, DTRSM then DGEMM above. */
static void trsm_upper_nonunit(int m, int n, const double* U, int ldu, double* B, int ldb) {
  const int kb = 32;
  int kmax = ((m - 1) / kb) * kb;
  for (int k = kmax; k >= 0; k -= kb) {
    blasint kbb = (m - k) < kb ? (m - k) : kb;
    blasint nn = n, l1 = ldu, l2 = ldb;
    p_dtrsm("L", "U", "N", "N", &kbb, &nn, &ONE, U + k + (size_t)k * ldu, &l1, B + k, &l2,
            1, 1, 1, 1);
    if (k > 0) {
      blasint kk = k;
      p_dgemm("N", "N", &kk, &nn, &kbb, &MONE, U + (size_t)k * ldu, &l1, B + k, &l2, &ONE, B, &l2,
              1, 1);
    }
  }
}

/* Transposed solves for PDGETRS TRANS='T'/'C' (SRC/pdgetrs.f:268-284),
 * blocked by 32 in the same way: U^T is lower (forward), L^T is upper
 * (backward). */
static void trsm_upperT_nonunit(int m, int n, const double* U, int ldu, double* B, int ldb) {
  const int kb = 32;
  for (int k = 0; k < m; k += kb) {
    blasint kbb = (m - k) < kb ? (m - k) : kb;
    blasint nn = n, l1 = ldu, l2 = ldb;
    p_dtrsm("L", "U", "T", "N", &kbb, &nn, &ONE, U + k + (size_t)k * ldu, &l1, B + k, &l2,
            1, 1, 1, 1);
    blasint rest = m - k - kbb;
    if (rest > 0)
      p_dgemm("T", "N", &rest, &nn, &kbb, &MONE, U + k + (size_t)(k + kbb) * ldu, &l1, B + k, &l2,
              &ONE, B + k + kbb, &l2, 1, 1);
  }
}
static void trsm_lowerT_unit(int m, int n, const double* L, int ldl, double* B, int ldb) {
  const int kb = 32;
  int kmax = ((m - 1) / kb) * kb;
  for (int k = kmax; k >= 0; k -= kb) {
    blasint kbb = (m - k) < kb ? (m - k) : kb;
    blasint nn = n, l1 = ldl, l2 = ldb;
    p_dtrsm("L", "L", "T", "U", &kbb, &nn, &ONE, L + k + (size_t)k * ldl, &l1, B + k, &l2,
            1, 1, 1, 1);
    if (k > 0) {
      blasint kk = k;
      p_dgemm("T", "N", &kk, &nn, &kbb, &MONE, L + k, &l1, B + k, &l2, &ONE, B, &l2, 1, 1);
    }
  }
}

/*
 * PDGETRF on a 1x1 grid (SRC/pdgetrf.f:199-302).  A is the local array with
 * leading dimension lda (= LLD_A); (ia, ja) is the 1-based origin of sub(A);
 * nb = NB_A (= MB_A); ipiv is the local IPIV (indexed by global row).
 * Returns INFO > 0 for the first exactly-zero pivot, 0 otherwise.
 * `mglob` is DESCA(M_) (the quick return at pdgetrf.f:201 tests it).
 */
int orc_pdgetrf(int m, int n, double* A, int lda, int ia, int ja, int nb, int mglob, int* ipiv) {
  if (mglob == 1) { ipiv[0] = 1; return 0; }
  if (m == 0 || n == 0) return 0;
  int info = 0;
  int mn = m < n ? m : n;
  /* ICEIL(IA,MB)*MB etc. (pdgetrf.f:219-221) */
  int in = ((ia + nb - 1) / nb) * nb; if (in > ia + m - 1) in = ia + m - 1;
  int jn = ((ja + nb - 1) / nb) * nb; if (jn > ja + mn - 1) jn = ja + mn - 1;
  int jb = jn - ja + 1;
  info = pdgetf2_1x1(m, jb, A, lda, ia, ja, ipiv, 0);
  if (jb + 1 <= n) {
    pdlaswp_fwd_1x1(n - jb, A, lda, jn + 1, ia, in, ipiv);
    trsm_lower_unit(jb, n - jb, A_(ia, ja), lda, A_(ia, jn + 1), lda);
    if (jb + 1 <= m) {
      blasint mm = m - jb, nn = n - jb, kk = jb, ld = lda;
      p_dgemm("N", "N", &mm, &nn, &kk, &MONE, A_(in + 1, ja), &ld, A_(ia, jn + 1), &ld, &ONE,
              A_(in + 1, jn + 1), &ld, 1, 1);
    }
  }
  for (int j = jn + 1; j <= ja + mn - 1; j += nb) {
    int jbb = (mn - j + ja) < nb ? (mn - j + ja) : nb;
    int i = ia + j - ja;
    int iinfo = pdgetf2_1x1(m - j + ja, jbb, A, lda, i, j, ipiv, j - ja);
    if (info == 0 && iinfo > 0) info = iinfo + j - ja;
    pdlaswp_fwd_1x1(j - ja, A, lda, ja, i, i + jbb - 1, ipiv);
    if (j - ja + jbb + 1 <= n) {
      pdlaswp_fwd_1x1(n - j - jbb + ja, A, lda, j + jbb, i, i + jbb - 1, ipiv);
      trsm_lower_unit(jbb, n - j - jbb + ja, A_(i, j), lda, A_(i, j + jbb), lda);
      if (j - ja + jbb + 1 <= m) {
        blasint mm = m - j - jbb + ja, nn = n - j - jbb + ja, kk = jbb, ld = lda;
        p_dgemm("N", "N", &mm, &nn, &kk, &MONE, A_(i + jbb, j), &ld, A_(i, j + jbb), &ld, &ONE,
                A_(i + jbb, j + jbb), &ld, 1, 1);
      }
    }
  }
  return info;
}

/*
 * PDGETRS on a 1x1 grid (SRC/pdgetrs.f:238-284).  trans: 'N', 'T' or 'C'.
 * B has leading dimension ldb with sub(B) at (ib, jb); A's factors at (ia, ja).
 * PDLAPIV forward (SRC/pdlapv2.f:208-242): row K of sub(B) is swapped with row
 * IPIV(IA+K-IB) - IA + IB.
 */
void orc_pdgetrs(char trans, int n, int nrhs, const double* A, int lda, int ia, int ja,
                 const int* ipiv, double* B, int ldb, int ib, int jb) {
  if (n == 0 || nrhs == 0) return;
  const double* Asub = A + (ia - 1) + (size_t)(ja - 1) * lda;
  double* Bsub = B + (ib - 1) + (size_t)(jb - 1) * ldb;
  blasint nn = nrhs, ld = ldb;
  int notran = (trans == 'N' || trans == 'n');
  if (notran) {
    for (int k = 0; k < n; ++k) {
      int p = ipiv[ia - 1 + k] - ia; /* 0-based row within sub(B) */
      if (p != k) p_dswap(&nn, Bsub + k, &ld, Bsub + p, &ld);
    }
    trsm_lower_unit(n, nrhs, Asub, lda, Bsub, ldb);
    trsm_upper_nonunit(n, nrhs, Asub, lda, Bsub, ldb);
  } else {
    trsm_upperT_nonunit(n, nrhs, Asub, lda, Bsub, ldb);
    trsm_lowerT_unit(n, nrhs, Asub, lda, Bsub, ldb);
    for (int k = n - 1; k >= 0; --k) {
      int p = ipiv[ia - 1 + k] - ia;
      if (p != k) p_dswap(&nn, Bsub + k, &ld, Bsub + p, &ld);
    }
  }
}

/* LAPACK DGETRF/DGETRS from the bound library (for pinning the restatement).
 * Returns -999 when no library routine is bound. */
int orc_lapack_dgetrf(int m, int n, double* A, int lda, int* ipiv) {
  if (!p_dgetrf) return -999;
  blasint mm = m, nn = n, ld = lda, info = 0;
  p_dgetrf(&mm, &nn, A, &ld, ipiv, &info);
  return info;
}
int orc_lapack_dgetrs(char trans, int n, int nrhs, const double* A, int lda, const int* ipiv,
                      double* B, int ldb) {
  if (!p_dgetrs) return -999;
  blasint nn = n, nr = nrhs, la = lda, lb = ldb, info = 0;
  char t[2] = {trans, 0};
  p_dgetrs(t, &nn, &nr, A, &la, ipiv, B, &lb, &info, 1);
  return info;
}

/* General dgemm passthrough (used for residuals by the Python side). */
void orc_dgemm(char ta, char tb, int m, int n, int k, double alpha, const double* a, int lda,
               const double* b, int ldb, double beta, double* c, int ldc) {
  blasint mm = m, nn = n, kk = k, l1 = lda, l2 = ldb, l3 = ldc;
  char s1[2] = {ta, 0}, s2[2] = {tb, 0};
  p_dgemm(s1, s2, &mm, &nn, &kk, &alpha, a, &l1, b, &l2, &beta, c, &l3, 1, 1);
}

/* ------------------------------------------------------------------------- */
/* Residual checks (tester semantics)                                         */
/* ------------------------------------------------------------------------- */
/* ||X||_inf of an m x n column-major block (PDLANGE 'I'). */
double orc_norm_inf(int m, int n, const double* X, int ldx) {
  double best = 0.0;
  double* rs = (double*)calloc((size_t)(m > 0 ? m : 1), sizeof(double));
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) rs[i] += fabs(X[i + (size_t)j * ldx]);
  for (int i = 0; i < m; ++i) if (rs[i] > best || isnan(rs[i])) best = rs[i];
  free(rs);
  return best;
}

/* eps as PDLAMCH('E') returns it: DLAMCH('E') = 2^-53 (rounding arithmetic). */
double orc_eps(void) { return ldexp(1.0, -53); }

/*
 * PDLASCHK (TESTING/traditional/LIN/pdlaschk.f:182-323) on a 1x1 grid:
 * RESID = max_j ||b_j - A x_j||_inf / (||x_j||_inf * ||A||_inf * eps * N).
 * A0 (n x n, lda0) and B0 (n x nrhs, ldb0) are the original inputs, X the
 * computed solution.
 */
double orc_sresid(int n, int nrhs, const double* A0, int lda0, const double* B0, int ldb0,
                  const double* X, int ldx, double anorm) {
  double* R = (double*)malloc(sizeof(double) * (size_t)n * (nrhs > 0 ? nrhs : 1));
  for (int j = 0; j < nrhs; ++j)
    for (int i = 0; i < n; ++i) R[i + (size_t)j * n] = B0[i + (size_t)j * ldb0];
  orc_dgemm('N', 'N', n, nrhs, n, -1.0, A0, lda0, X, ldx, 1.0, R, n);
  double divisor = anorm * orc_eps() * (double)n;
  double resid = 0.0;
  for (int j = 0; j < nrhs; ++j) {
    double rmax = 0.0, xmax = 0.0;
    for (int i = 0; i < n; ++i) {
      double r = fabs(R[i + (size_t)j * n]), x = fabs(X[i + (size_t)j * ldx]);
      if (r > rmax || isnan(r)) rmax = r;
      if (x > xmax || isnan(x)) xmax = x;
    }
    double r1 = rmax / (xmax * divisor);
    if (resid < r1 || isnan(r1)) resid = r1;
  }
  free(R);
  return resid;
}

/*
 * PDGETRRV + PDLAFCHK (LIN/pdgetrrv.f:210-289, LIN/pdlafchk.f:182-226):
 * FRESID = ||P*L*U - A||_inf / (max(M,N) * eps * ||A||_inf).
 * LU (m x n, ldlu) holds the factors, ipiv the 1-based pivots of sub(A)
 * (relative: row k was swapped with ipiv[k]).
 */
double orc_fresid(int m, int n, const double* LU, int ldlu, const int* ipiv_rel, const double* A0,
                  int lda0, double anorm) {
  int mn = m < n ? m : n;
  double* L = (double*)calloc((size_t)m * mn, sizeof(double));
  double* U = (double*)calloc((size_t)mn * n, sizeof(double));
  double* R = (double*)malloc(sizeof(double) * (size_t)m * n);
  for (int j = 0; j < mn; ++j)
    for (int i = 0; i < m; ++i) {
      if (i == j) L[i + (size_t)j * m] = 1.0;
      else if (i > j) L[i + (size_t)j * m] = LU[i + (size_t)j * ldlu];
    }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i <= j && i < mn; ++i) U[i + (size_t)j * mn] = LU[i + (size_t)j * ldlu];
  orc_dgemm('N', 'N', m, n, mn, 1.0, L, m, U, mn, 0.0, R, m);
  /* apply P: undo the swaps in reverse order (PDGETRRV applies the inverse
   * row interchanges to L*U). */
  for (int k = mn - 1; k >= 0; --k) {
    int p = ipiv_rel[k] - 1;
    if (p != k)
      for (int j = 0; j < n; ++j) {
        double t = R[k + (size_t)j * m];
        R[k + (size_t)j * m] = R[p + (size_t)j * m];
        R[p + (size_t)j * m] = t;
      }
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) R[i + (size_t)j * m] -= A0[i + (size_t)j * lda0];
  double num = orc_norm_inf(m, n, R, m);
  free(L); free(U); free(R);
  int mx = m > n ? m : n;
  return num / ((double)mx * orc_eps() * anorm);
}

/* ------------------------------------------------------------------------- */
/* Conditioned generator (pattern of TOOLS/LAPACK/dlagge.f:115-165)            */
/* ------------------------------------------------------------------------- */
/* A = (H_1 ... H_r) diag(s) (G_1 ... G_r)^T with r seeded Householder
 * reflectors H = I - 2 v v^T / (v^T v) per side and s geometric from 1 to
 * 1/kappa.  Reflector vectors come from the PDMATGEN LCG (kind 1) with seeds
 * seed (left) and seed+1 (right), one n-vector per reflector.  Plain loops:
 * intended for the moderate sizes the tests use. */
void orc_gen_conditioned(int n, int nrefl, double kappa, int seed, double* A, int lda) {
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) A[i + (size_t)j * lda] = 0.0;
  for (int i = 0; i < n; ++i)
    A[i + (size_t)i * lda] = (n == 1) ? 1.0 : pow(kappa, -(double)i / (double)(n - 1));
  double* v = (double*)malloc(sizeof(double) * (size_t)n);
  double* w = (double*)malloc(sizeof(double) * (size_t)n);
  for (int side = 0; side < 2; ++side) {
    for (int r = 0; r < nrefl; ++r) {
      orc_matgen(n, nrefl, seed + side, 1, 0, 0, r, n, 1, v, n);
      double vv = 0.0;
      for (int i = 0; i < n; ++i) vv += v[i] * v[i];
      double tau = 2.0 / vv;
      if (side == 0) { /* A <- (I - tau v v^T) A */
        for (int j = 0; j < n; ++j) {
          double s = 0.0;
          for (int i = 0; i < n; ++i) s += v[i] * A[i + (size_t)j * lda];
          w[j] = tau * s;
        }
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) A[i + (size_t)j * lda] -= v[i] * w[j];
      } else { /* A <- A (I - tau v v^T) */
        for (int i = 0; i < n; ++i) w[i] = 0.0;
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) w[i] += A[i + (size_t)j * lda] * v[j];
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) A[i + (size_t)j * lda] -= tau * w[i] * v[j];
      }
    }
  }
  free(v); free(w);
}

/* ------------------------------------------------------------------------- */
/* Expert driver: PDGEEQU, PDLAQGE, PDLACON, PDGECON, PDLANGE, PDGERFS,       */
/* PDGESVX on a 1x1 grid                                                      */
/* ------------------------------------------------------------------------- */
#define A_AT(M, ld, i, j) ((M)[(size_t)(i) + (size_t)(j) * (size_t)(ld)])
static const double ORC_SAFMIN = 2.2250738585072014e-308; /* 2^-1022, PDLAMCH 'S' */

/* PDGEEQU (SRC/pdgeequ.f:230-340) for sub(A) = A(ia.., ja..), m x n.
 * R[i] stands for R(IA+i) and C[j] for C(JA+j).  Returns INFO. */
int orc_pdgeequ(int m, int n, const double* A, int lda, int ia, int ja, double* R, double* C,
                double* rowcnd, double* colcnd, double* amax) {
  if (m == 0 || n == 0) { *rowcnd = 1.0; *colcnd = 1.0; *amax = 0.0; return 0; }
  const double* S = A + (ia - 1) + (size_t)(ja - 1) * lda;
  const double smlnum = ORC_SAFMIN, bignum = 1.0 / smlnum;
  for (int i = 0; i < m; ++i) R[i] = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) R[i] = fmax(R[i], fabs(A_AT(S, lda, i, j)));
  double rcmin = bignum, rcmax = 0.0;
  for (int i = 0; i < m; ++i) { rcmax = fmax(rcmax, R[i]); rcmin = fmin(rcmin, R[i]); }
  *amax = rcmax;
  if (rcmin == 0.0) {
    for (int i = 0; i < m; ++i) if (R[i] == 0.0) return i + 1;
  }
  for (int i = 0; i < m; ++i) R[i] = 1.0 / fmin(fmax(R[i], smlnum), bignum);
  *rowcnd = fmax(rcmin, smlnum) / fmin(rcmax, bignum);
  for (int j = 0; j < n; ++j) C[j] = 0.0;
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) C[j] = fmax(C[j], fabs(A_AT(S, lda, i, j)) * R[i]);
  rcmin = bignum; rcmax = 0.0;
  for (int j = 0; j < n; ++j) { rcmin = fmin(rcmin, C[j]); rcmax = fmax(rcmax, C[j]); }
  if (rcmin == 0.0) {
    for (int j = 0; j < n; ++j) if (C[j] == 0.0) return m + j + 1;
  }
  for (int j = 0; j < n; ++j) C[j] = 1.0 / fmin(fmax(C[j], smlnum), bignum);
  *colcnd = fmax(rcmin, smlnum) / fmin(rcmax, bignum);
  return 0;
}

/* PDLAQGE (SRC/pdlaqge.f:180-260).  Returns EQUED. */
char orc_pdlaqge(int m, int n, double* A, int lda, int ia, int ja, const double* R,
                 const double* C, double rowcnd, double colcnd, double amax) {
  if (m <= 0 || n <= 0) return 'N';
  double* S = A + (ia - 1) + (size_t)(ja - 1) * lda;
  const double small = ORC_SAFMIN / ldexp(1.0, -52); /* 'Safe minimum' / 'Precision' */
  const double large = 1.0 / small, thresh = 0.1;
  if (rowcnd >= thresh && amax >= small && amax <= large) {
    if (colcnd >= thresh) return 'N';
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) A_AT(S, lda, i, j) = C[j] * A_AT(S, lda, i, j);
    return 'C';
  }
  if (colcnd >= thresh) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < m; ++i) A_AT(S, lda, i, j) = R[i] * A_AT(S, lda, i, j);
    return 'R';
  }
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < m; ++i) A_AT(S, lda, i, j) = C[j] * R[i] * A_AT(S, lda, i, j);
  return 'B';
}

/* Hager/Higham 1-norm estimator as PDLACON (SRC/pdlacon.f) runs it on one
 * process: op(1, x) overwrites x with B x, op(2, x) with B^T x. */
typedef void (*orc_op_t)(int kase, double* x, void* ctx);
static double orc_dlacon(int n, orc_op_t op, void* ctx) {
  double* x = (double*)malloc(sizeof(double) * (size_t)n);
  int* isgn = (int*)malloc(sizeof(int) * (size_t)n);
  double est = 0.0;
  for (int i = 0; i < n; ++i) x[i] = 1.0 / n;
  op(1, x, ctx);
  if (n == 1) { est = fabs(x[0]); free(x); free(isgn); return est; }
  for (int i = 0; i < n; ++i) est += fabs(x[i]);
  for (int i = 0; i < n; ++i) { x[i] = x[i] >= 0.0 ? 1.0 : -1.0; isgn[i] = (int)x[i]; }
  op(2, x, ctx);
  int j = 0;
  for (int i = 1; i < n; ++i) if (fabs(x[i]) > fabs(x[j])) j = i;
  int iter = 2;
  for (;;) {
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    x[j] = 1.0;
    op(1, x, ctx);
    const double estold = est;
    est = 0.0;
    for (int i = 0; i < n; ++i) est += fabs(x[i]);
    int changed = 0;
    for (int i = 0; i < n; ++i) if ((x[i] >= 0.0 ? 1 : -1) != isgn[i]) { changed = 1; break; }
    if (!changed || est <= estold) break;
    for (int i = 0; i < n; ++i) { x[i] = x[i] >= 0.0 ? 1.0 : -1.0; isgn[i] = (int)x[i]; }
    op(2, x, ctx);
    const int jlast = j;
    j = 0;
    for (int i = 1; i < n; ++i) if (fabs(x[i]) > fabs(x[j])) j = i;
    if (x[jlast] == fabs(x[j]) || iter >= 5) break;
    ++iter;
  }
  double altsgn = 1.0;
  for (int i = 0; i < n; ++i) { x[i] = altsgn * (1.0 + (double)i / (double)(n - 1)); altsgn = -altsgn; }
  op(1, x, ctx);
  double temp = 0.0;
  for (int i = 0; i < n; ++i) temp += fabs(x[i]);
  temp = 2.0 * temp / (3.0 * n);
  if (temp > est) est = temp;
  free(x); free(isgn);
  return est;
}

/* PDLANGE '1' (max column sum) or 'I' (max row sum) of sub(A), n x n. */
double orc_pdlange(char norm, int n, const double* A, int lda, int ia, int ja) {
  const double* S = A + (ia - 1) + (size_t)(ja - 1) * lda;
  double v = 0.0;
  if (norm == '1' || norm == 'O' || norm == 'o') {
    for (int j = 0; j < n; ++j) {
      double s = 0.0;
      for (int i = 0; i < n; ++i) s += fabs(A_AT(S, lda, i, j));
      if (s > v) v = s;
    }
  } else {
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int j = 0; j < n; ++j) s += fabs(A_AT(S, lda, i, j));
      if (s > v) v = s;
    }
  }
  return v;
}

struct orc_inv_ctx { int n; const double* LU; int ld; int onenrm; };
static void orc_gecon_op(int kase, double* x, void* vctx) {
  struct orc_inv_ctx* c = (struct orc_inv_ctx*)vctx;
  const int kase1 = c->onenrm ? 1 : 2;
  if (kase == kase1) { /* inv(U) inv(L) x */
    trsm_lower_unit(c->n, 1, c->LU, c->ld, x, c->n);
    trsm_upper_nonunit(c->n, 1, c->LU, c->ld, x, c->n);
  } else {             /* inv(L)^T inv(U)^T x */
    trsm_upperT_nonunit(c->n, 1, c->LU, c->ld, x, c->n);
    trsm_lowerT_unit(c->n, 1, c->LU, c->ld, x, c->n);
  }
}

/* PDGECON (SRC/pdgecon.f) with unscaled triangular solves. */
double orc_pdgecon(char norm, int n, const double* AF, int ldaf, int iaf, int jaf, double anorm) {
  if (n == 0) return 1.0;
  if (anorm == 0.0) return 0.0;
  struct orc_inv_ctx c = {n, AF + (iaf - 1) + (size_t)(jaf - 1) * ldaf, ldaf,
                          (norm == '1' || norm == 'O' || norm == 'o')};
  const double ainvnm = orc_dlacon(n, orc_gecon_op, &c);
  return ainvnm != 0.0 ? (1.0 / ainvnm) / anorm : 0.0;
}

struct orc_rfs_ctx {
  char trans, transt;
  int n; const double* AF; int ldaf, iaf, jaf; const int* ipiv; const double* w;
};
static void orc_rfs_op(int kase, double* x, void* vctx) {
  struct orc_rfs_ctx* c = (struct orc_rfs_ctx*)vctx;
  if (kase == 1) { /* diag(W) inv(op(A))^T */
    orc_pdgetrs(c->transt, c->n, 1, c->AF, c->ldaf, c->iaf, c->jaf, c->ipiv, x, c->n, 1, 1);
    for (int i = 0; i < c->n; ++i) x[i] = c->w[i] * x[i];
  } else {         /* inv(op(A)) diag(W) */
    for (int i = 0; i < c->n; ++i) x[i] = c->w[i] * x[i];
    orc_pdgetrs(c->trans, c->n, 1, c->AF, c->ldaf, c->iaf, c->jaf, c->ipiv, x, c->n, 1, 1);
  }
}

/* PDGERFS (SRC/pdgerfs.f:470-887) on a 1x1 grid.  ferr[k] / berr[k] stand for
 * FERR(JB+k) / BERR(JB+k); ferr[k] is left as it was when column k of X is 0. */
void orc_pdgerfs(char trans, int n, int nrhs, const double* A, int lda, int ia, int ja,
                 const double* AF, int ldaf, int iaf, int jaf, const int* ipiv, const double* B,
                 int ldb, int ib, int jb, double* X, int ldx, int ix, int jx, double* ferr,
                 double* berr) {
  if (n <= 1 || nrhs == 0) {
    for (int k = 0; k < nrhs; ++k) { ferr[k] = 0.0; berr[k] = 0.0; }
    return;
  }
  const int notran = (trans == 'N' || trans == 'n');
  const double* SA = A + (ia - 1) + (size_t)(ja - 1) * lda;
  const int nz = n + 1;
  const double eps = orc_eps();
  const double safe1 = nz * ORC_SAFMIN, safe2 = safe1 / eps;
  double* r = (double*)malloc(sizeof(double) * (size_t)n);
  double* w = (double*)malloc(sizeof(double) * (size_t)n);
  for (int k = 0; k < nrhs; ++k) {
    const double* b = B + (ib - 1) + (size_t)(jb - 1 + k) * ldb;
    double* x = X + (ix - 1) + (size_t)(jx - 1 + k) * ldx;
    int count = 1;
    double lstres = 3.0;
    for (;;) {
      /* r = b - op(A) x, w = |b| + |op(A)| |x| */
      for (int i = 0; i < n; ++i) { r[i] = b[i]; w[i] = fabs(b[i]); }
      if (notran) {
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) {
            r[i] -= A_AT(SA, lda, i, j) * x[j];
            w[i] += fabs(A_AT(SA, lda, i, j)) * fabs(x[j]);
          }
      } else {
        for (int j = 0; j < n; ++j) {
          double s = 0.0, t = 0.0;
          for (int i = 0; i < n; ++i) {
            s += A_AT(SA, lda, i, j) * x[i];
            t += fabs(A_AT(SA, lda, i, j)) * fabs(x[i]);
          }
          r[j] -= s;
          w[j] += t;
        }
      }
      double s = 0.0;
      for (int i = 0; i < n; ++i) {
        const double q = (w[i] > safe2) ? fabs(r[i]) / w[i] : (fabs(r[i]) + safe1) / (w[i] + safe1);
        if (q > s) s = q;
      }
      berr[k] = s;
      if (s > eps && 2.0 * s <= lstres && count <= 5) {
        orc_pdgetrs(trans, n, 1, AF, ldaf, iaf, jaf, ipiv, r, n, 1, 1);
        for (int i = 0; i < n; ++i) x[i] = x[i] + r[i];
        lstres = s;
        ++count;
        continue;
      }
      break;
    }
    for (int i = 0; i < n; ++i)
      w[i] = (w[i] > safe2) ? fabs(r[i]) + nz * eps * w[i] : fabs(r[i]) + nz * eps * w[i] + safe1;
    struct orc_rfs_ctx c = {notran ? 'N' : 'T', notran ? 'T' : 'N', n, AF, ldaf, iaf, jaf, ipiv, w};
    const double est = orc_dlacon(n, orc_rfs_op, &c);
    double xmax = 0.0;
    for (int i = 0; i < n; ++i) xmax = fmax(xmax, fabs(x[i]));
    if (xmax != 0.0) ferr[k] = est / xmax;
  }
  free(r); free(w);
}

/* PDGESVX (SRC/pdgesvx.f:660-845) on a 1x1 grid, after argument checks.
 * R[i] is R(i+1) and C[j] is C(j+1) (full local arrays); ferr/berr are the
 * full FERR/BERR arrays (FERR(j) = ferr[j-1]).  With FACT = 'F', TRANS = 'N'
 * and column equilibration, X is multiplied by C (the reference multiplies by
 * a workspace it never filled there).  mglob_af is DESCAF(M_), nb = NB_AF.
 * Returns INFO. */
int orc_pdgesvx(char fact, char trans, int n, int nrhs, double* A, int lda, int ia, int ja,
                double* AF, int ldaf, int iaf, int jaf, int mglob_af, int nb, int* ipiv,
                char* equed, double* R, double* C, double* B, int ldb, int ib, int jb, double* X,
                int ldx, int ix, int jx, double* rcond, double* ferr, double* berr) {
  const int nofact = (fact == 'N'), equil = (fact == 'E'), notran = (trans == 'N');
  int rowequ = 0, colequ = 0;
  double rowcnd = 1.0, colcnd = 1.0;
  const double smlnum = ORC_SAFMIN, bignum = 1.0 / smlnum;
  if (nofact || equil) {
    *equed = 'N';
  } else {
    rowequ = (*equed == 'R' || *equed == 'B');
    colequ = (*equed == 'C' || *equed == 'B');
    if (rowequ) {
      double mn = bignum, mx = 0.0;
      for (int i = 0; i < n; ++i) { mn = fmin(mn, R[ia - 1 + i]); mx = fmax(mx, R[ia - 1 + i]); }
      rowcnd = n > 0 ? fmax(mn, smlnum) / fmin(mx, bignum) : 1.0;
    }
    if (colequ) {
      double mn = bignum, mx = 0.0;
      for (int j = 0; j < n; ++j) { mn = fmin(mn, C[ja - 1 + j]); mx = fmax(mx, C[ja - 1 + j]); }
      colcnd = n > 0 ? fmax(mn, smlnum) / fmin(mx, bignum) : 1.0;
    }
  }
  if (n == 0) {
    *rcond = 1.0;
    for (int k = 0; k < nrhs; ++k) { ferr[jb - 1 + k] = 0.0; berr[jb - 1 + k] = 0.0; }
    return 0;
  }
  /* 1. equilibrate */
  if (equil) {
    double rc = 1.0, cc = 1.0, amax = 0.0;
    const int infequ = orc_pdgeequ(n, n, A, lda, ia, ja, R + (ia - 1), C + (ja - 1), &rc, &cc, &amax);
    if (infequ == 0) {
      rowcnd = rc;
      colcnd = cc;
      *equed = orc_pdlaqge(n, n, A, lda, ia, ja, R + (ia - 1), C + (ja - 1), rowcnd, colcnd, amax);
      rowequ = (*equed == 'R' || *equed == 'B');
      colequ = (*equed == 'C' || *equed == 'B');
    }
  }
  /* scale B: R(IB..) rows (op = N) or C(JA..) (op = T) */
  if (notran ? rowequ : colequ) {
    for (int k = 0; k < nrhs; ++k)
      for (int i = 0; i < n; ++i) {
        const double v = notran ? R[ib - 1 + i] : C[ja - 1 + i];
        A_AT(B, ldb, ib - 1 + i, jb - 1 + k) = v * A_AT(B, ldb, ib - 1 + i, jb - 1 + k);
      }
  }
  /* 2. factor */
  if (nofact || equil) {
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        A_AT(AF, ldaf, iaf - 1 + i, jaf - 1 + j) = A_AT(A, lda, ia - 1 + i, ja - 1 + j);
    const int info = orc_pdgetrf(n, n, AF, ldaf, iaf, jaf, nb, mglob_af, ipiv);
    if (info != 0) {
      if (info > 0) *rcond = 0.0;
      return info;
    }
  }
  /* 3. condition estimate */
  const char norm = notran ? '1' : 'I';
  const double anorm = orc_pdlange(norm, n, A, lda, ia, ja);
  *rcond = orc_pdgecon(norm, n, AF, ldaf, iaf, jaf, anorm);
  if (*rcond < orc_eps()) return ia + n;
  /* 4. solve, 5. refine */
  for (int k = 0; k < nrhs; ++k)
    for (int i = 0; i < n; ++i)
      A_AT(X, ldx, ix - 1 + i, jx - 1 + k) = A_AT(B, ldb, ib - 1 + i, jb - 1 + k);
  orc_pdgetrs(notran ? 'N' : 'T', n, nrhs, AF, ldaf, iaf, jaf, ipiv, X, ldx, ix, jx);
  orc_pdgerfs(notran ? 'N' : 'T', n, nrhs, A, lda, ia, ja, AF, ldaf, iaf, jaf, ipiv, B, ldb, ib,
              jb, X, ldx, ix, jx, ferr + (jb - 1), berr + (jb - 1));
  /* 6. back to the original system */
  if (notran ? colequ : rowequ) {
    const double cnd = notran ? colcnd : rowcnd;
    for (int k = 0; k < nrhs; ++k) {
      for (int i = 0; i < n; ++i) {
        const double v = notran ? C[ja - 1 + i] : R[ix - 1 + i];
        A_AT(X, ldx, ix - 1 + i, jx - 1 + k) = v * A_AT(X, ldx, ix - 1 + i, jx - 1 + k);
      }
      ferr[jx - 1 + k] = ferr[jx - 1 + k] / cnd;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------------- */
/* PDGETRI on a 1x1 grid                                                      */
/* ------------------------------------------------------------------------- */
/* PDTRTI2, upper non-unit (SRC/pdtrti2.f:194-211), on the n x n block T (ld
 * ldt): column j's diagonal is inverted, then its entries above the diagonal
 * become -inv(T(j,j)) times the already-inverted leading block applied to
 * them (DTRMV 'Upper', in place, rows in ascending order). */
static void orc_trti2_upper(int n, double* T, int ldt) {
  for (int j = 0; j < n; ++j) {
    A_AT(T, ldt, j, j) = 1.0 / A_AT(T, ldt, j, j);
    const double ajj = -A_AT(T, ldt, j, j);
    for (int i = 0; i < j; ++i) {
      double s = 0.0;
      for (int k = i; k < j; ++k) s += A_AT(T, ldt, i, k) * A_AT(T, ldt, k, j);
      A_AT(T, ldt, i, j) = s;
    }
    for (int i = 0; i < j; ++i) A_AT(T, ldt, i, j) *= ajj;
  }
}

/* PDGETRI (SRC/pdgetri.f:299-372) with PDTRTRI (SRC/pdtrtri.f:226-302) on a
 * 1x1 grid: A (n x n at (ia, ja), ld lda) holds L\U and ipiv_rel the 0-based
 * pivot rows relative to IA. Returns INFO: the first zero U(i,i) (1-based;
 * A untouched) or 0 with inv(A) in place. Blocked by nb as the reference:
 * inv(U) block column by block column (TRMM with the inverted leading block,
 * TRSM by the diagonal block, PDTRTI2 on it), then inv(A) L = inv(U) from the
 * last block column back (the block column of L copied out and zeroed, one
 * GEMM with the columns already done, a unit-lower TRSM from the right), then
 * the pivots applied to the columns backwards (PDLAPIV 'Backward', 'Columns'). */
int orc_pdgetri(int n, double* A, int lda, int ia, int ja, const int* ipiv_rel, int nb) {
  if (n <= 0) return 0;
  double* S = A + (ia - 1) + (size_t)(ja - 1) * lda;
  for (int i = 0; i < n; ++i)
    if (A_AT(S, lda, i, i) == 0.0) return i + 1;
  if (nb < 1) nb = 1;
  /* inv(U) */
  for (int j = 0; j < n; j += nb) {
    const int jb = (n - j) < nb ? (n - j) : nb;
    if (j > 0) {
      /* B = A(0:j, j:j+jb) := triu(A(0:j, 0:j)) B (TRMM 'Left', 'Upper'): row by row ascending */
      for (int c = 0; c < jb; ++c)
        for (int i = 0; i < j; ++i) {
          double s = 0.0;
          for (int k = i; k < j; ++k) s += A_AT(S, lda, i, k) * A_AT(S, lda, k, j + c);
          A_AT(S, lda, i, j + c) = s;
        }
      /* B := -B inv(U_jj) (TRSM 'Right', 'Upper', non-unit): columns ascending */
      for (int c = 0; c < jb; ++c) {
        for (int k = 0; k < c; ++k) {
          const double u = A_AT(S, lda, j + k, j + c);
          for (int i = 0; i < j; ++i) A_AT(S, lda, i, j + c) -= A_AT(S, lda, i, j + k) * u;
        }
        const double d = A_AT(S, lda, j + c, j + c);
        for (int i = 0; i < j; ++i) A_AT(S, lda, i, j + c) /= d;
      }
      for (int c = 0; c < jb; ++c)
        for (int i = 0; i < j; ++i) A_AT(S, lda, i, j + c) = -A_AT(S, lda, i, j + c);
    }
    orc_trti2_upper(jb, &A_AT(S, lda, j, j), lda);
  }
  /* inv(A) L = inv(U), block columns from the last one back */
  double* W = (double*)malloc(sizeof(double) * (size_t)n * (size_t)nb);
  const int nn = ((n - 1) / nb) * nb;
  for (int j = nn; j >= 0; j -= nb) {
    const int jb = (n - j) < nb ? (n - j) : nb;
    /* W(r, c) = L(r, j + c) for rows r > j + c (W is n x jb, row index global), then zeroed in A */
    for (int c = 0; c < jb; ++c)
      for (int r = 0; r < n; ++r) {
        if (r > j + c) {
          A_AT(W, n, r, c) = A_AT(S, lda, r, j + c);
          A_AT(S, lda, r, j + c) = 0.0;
        } else {
          A_AT(W, n, r, c) = 0.0;
        }
      }
    if (j + jb < n)
      orc_dgemm('N', 'N', n, jb, n - j - jb, -1.0, &A_AT(S, lda, 0, j + jb), lda, &A_AT(W, n, j + jb, 0),
                n, 1.0, &A_AT(S, lda, 0, j), lda);
    /* X(:, j:j+jb) := X inv(L_jj) (TRSM 'Right', 'Lower', unit): columns descending */
    for (int c = jb - 1; c >= 0; --c)
      for (int k = c + 1; k < jb; ++k) {
        const double l = A_AT(W, n, j + k, c);
        for (int i = 0; i < n; ++i) A_AT(S, lda, i, j + c) -= A_AT(S, lda, i, j + k) * l;
      }
  }
  free(W);
  /* the row interchanges of the factorization, applied to the columns backwards */
  for (int j = n - 1; j >= 0; --j) {
    const int p = ipiv_rel[j];
    if (p != j)
      for (int i = 0; i < n; ++i) {
        const double t = A_AT(S, lda, i, j);
        A_AT(S, lda, i, j) = A_AT(S, lda, i, p);
        A_AT(S, lda, i, p) = t;
      }
  }
  return 0;
}
