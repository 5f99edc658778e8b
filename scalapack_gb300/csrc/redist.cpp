// Block-cyclic redistribution (the data-format step in front of the LU):
//
//   pdgemr2d_            PDGEMR2D (REDIST/SRC/pdgemr.c) for the contexts this
//                        library runs, 1x1 grids: a submatrix copy between two
//                        descriptors (different block sizes, offsets and LLD).
//   sl1x1_redist_count / _pack / _unpack
//                        the per-process-pair pieces of a redistribution
//                        between two 2D block-cyclic layouts on any P0 x Q0 and
//                        P1 x Q1 grids. A transport that moves one buffer per
//                        (source, destination) pair -- an MPI all-to-all, or
//                        torch.distributed (scalapack_gb300/redist.py) --
//                        completes PDGEMR2D between processes.
//
// Canonical order of a (source, destination) buffer: the elements of
// sub(A) = A(IA:IA+M-1, JA:JA+N-1) that the source owns in A's layout and the
// destination owns in B's layout (sub(B) = B(IB:IB+M-1, JB:JB+N-1)),
// column-major in the submatrix's own coordinates. Both sides enumerate the
// same list, so no indices travel with the data. The reference reaches the
// same element sets through its interval intersections (block2buff /
// buff2block in REDIST/SRC/pdgemr.c); only the wire order differs.
#include <cstdio>
#include <mutex>
#include <vector>

#include "../../include/sl1x1.h"
#include "host_state.h"

using namespace sl::host;

namespace {

// Rows (or columns) r in [0, m) of the submatrix owned by process `ps` of A's
// p0 grid dimension and by `pd` of B's p1 grid dimension, with their local
// indices on each side (0-based). Distribution along one dimension: global
// index g is owned by (src + g / nb) mod p, at local (g / (nb p)) nb + g mod nb.
struct Axis {
  std::vector<long long> la, lb;
};

Axis intersect(int m, int i0a, int nba, int srca, int pa, int ps, int i0b, int nbb, int srcb,
               int pb, int pd) {
  Axis ax;
  if (ps < 0 || pd < 0) return ax;
  for (int r = 0; r < m; ++r) {
    const long long ga = (long long)i0a - 1 + r;
    const long long gb = (long long)i0b - 1 + r;
    if ((srca + ga / nba) % pa != ps) continue;
    if ((srcb + gb / nbb) % pb != pd) continue;
    ax.la.push_back((ga / ((long long)nba * pa)) * nba + ga % nba);
    ax.lb.push_back((gb / ((long long)nbb * pb)) * nbb + gb % nbb);
  }
  return ax;
}

struct Pair {
  Axis rows, cols;
  long long count() const { return (long long)rows.la.size() * (long long)cols.la.size(); }
};

Pair make_pair_(int m, int n, int ia, int ja, const int* desca, int p0, int q0, int sr, int sc,
                int ib, int jb, const int* descb, int p1, int q1, int dr, int dc) {
  Pair p;
  p.rows = intersect(m, ia, desca[MB_], desca[RSRC_], p0, sr, ib, descb[MB_], descb[RSRC_], p1, dr);
  p.cols = intersect(n, ja, desca[NB_], desca[CSRC_], q0, sc, jb, descb[NB_], descb[CSRC_], q1, dc);
  return p;
}

bool sane(int m, int n, const int* d, int p, int q) {
  return m >= 0 && n >= 0 && p >= 1 && q >= 1 && d[MB_] >= 1 && d[NB_] >= 1 && d[RSRC_] >= 0 &&
         d[RSRC_] < p && d[CSRC_] >= 0 && d[CSRC_] < q && d[LLD_] >= 1;
}

}  // namespace

extern "C" {

long long sl1x1_redist_count(int m, int n, int ia, int ja, const int* desca, int p0, int q0,
                             int sr, int sc, int ib, int jb, const int* descb, int p1, int q1,
                             int dr, int dc) {
  if (!sane(m, n, desca, p0, q0) || !sane(m, n, descb, p1, q1)) return -1;
  return make_pair_(m, n, ia, ja, desca, p0, q0, sr, sc, ib, jb, descb, p1, q1, dr, dc).count();
}

long long sl1x1_redist_pack(int m, int n, int ia, int ja, const int* desca, int p0, int q0, int sr,
                            int sc, int ib, int jb, const int* descb, int p1, int q1, int dr,
                            int dc, const double* A, double* buf) {
  if (!sane(m, n, desca, p0, q0) || !sane(m, n, descb, p1, q1)) return -1;
  const Pair p = make_pair_(m, n, ia, ja, desca, p0, q0, sr, sc, ib, jb, descb, p1, q1, dr, dc);
  const long long lda = desca[LLD_];
  long long k = 0;
  for (long long cj : p.cols.la)
    for (long long ri : p.rows.la) buf[k++] = A[ri + cj * lda];
  return k;
}

long long sl1x1_redist_unpack(int m, int n, int ia, int ja, const int* desca, int p0, int q0,
                              int sr, int sc, int ib, int jb, const int* descb, int p1, int q1,
                              int dr, int dc, const double* buf, double* B) {
  if (!sane(m, n, desca, p0, q0) || !sane(m, n, descb, p1, q1)) return -1;
  const Pair p = make_pair_(m, n, ia, ja, desca, p0, q0, sr, sc, ib, jb, descb, p1, q1, dr, dc);
  const long long ldb = descb[LLD_];
  long long k = 0;
  for (long long cj : p.cols.lb)
    for (long long ri : p.rows.lb) B[ri + cj * ldb] = buf[k++];
  return k;
}

// PDGEMR2D on the contexts of this library (1x1 grids). A process outside a
// context passes CTXT = -1 for it (as the reference asks); with both contexts
// 1x1 the call copies sub(A) into sub(B). Argument errors print a message
// and return without copying (the reference prints and exits the program).
void pdgemr2d_(const int* M, const int* N, const double* A, const int* IA, const int* JA,
               const int* DESCA, double* B, const int* IB, const int* JB, const int* DESCB,
               const int* ICTXT) {
  (void)ICTXT;
  const int m = *M, n = *N;
  if (m == 0 || n == 0) return;
  int pa, qa, ra, ca, pb, qb, rb, cb;
  gridinfo(DESCA[CTXT_], &pa, &qa, &ra, &ca);
  gridinfo(DESCB[CTXT_], &pb, &qb, &rb, &cb);
  const bool in_a = (DESCA[CTXT_] != -1 && pa == 1);
  const bool in_b = (DESCB[CTXT_] != -1 && pb == 1);
  auto bad = [&](const char* what) {
    std::fprintf(stderr, "PDGEMR2D: %s; nothing was copied\n", what);
  };
  if (m < 0 || n < 0) return bad("M or N is negative");
  if (!in_a || !in_b) {
    if ((DESCA[CTXT_] != -1 && !in_a) || (DESCB[CTXT_] != -1 && !in_b))
      return bad("a context is not a 1x1 grid of this process");
    return;  // this process holds neither side's data
  }
  // paramcheck (REDIST/SRC/pgemraux.c): the submatrix must lie in each matrix
  if (*IA < 1 || *JA < 1 || *IA + m - 1 > DESCA[M_] || *JA + n - 1 > DESCA[N_])
    return bad("sub(A) is out of A's bounds");
  if (*IB < 1 || *JB < 1 || *IB + m - 1 > DESCB[M_] || *JB + n - 1 > DESCB[N_])
    return bad("sub(B) is out of B's bounds");
  if (!sane(m, n, DESCA, 1, 1) || !sane(m, n, DESCB, 1, 1)) return bad("invalid descriptor");
  const long long lda = DESCA[LLD_], ldb = DESCB[LLD_];
  if (lda < DESCA[M_] || ldb < DESCB[M_]) return bad("LLD below the number of rows");
  // on one process both layouts are the identity: a strided submatrix copy
  for (int j = 0; j < n; ++j) {
    const double* src = A + (*IA - 1) + (long long)(*JA - 1 + j) * lda;
    double* dst = B + (*IB - 1) + (long long)(*JB - 1 + j) * ldb;
    for (int i = 0; i < m; ++i) dst[i] = src[i];
  }
}

}  // extern "C"
