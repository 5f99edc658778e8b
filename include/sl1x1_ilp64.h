/* sl1x1_ilp64.h -- the Fortran-ABI entry points of sl1x1.h for callers built
 * with 8-byte INTEGERs: the reference's "Int=long" build (README:145-154:
 * "-DInt=long" for C, "-fdefault-integer-8" / "-i8" for Fortran), which keeps
 * the routine names and changes every INTEGER argument, descriptor entry and
 * INTEGER array (IPIV, IWORK) to 8 bytes.
 *
 * Library: scalapack_gb300/_lib/libsl1x1gpu_ilp64.so, linked instead of
 * libsl1x1gpu.so; it loads libsl1x1gpu.so from its own directory (privately,
 * RTLD_LOCAL) and forwards every call. Each INTEGER is narrowed to 32 bits on
 * the way in and widened on the way out; the library's own index arithmetic
 * is 64-bit throughout (a 190 000 x 190 000 FP64 matrix, the largest that
 * fits the GPU's memory, has N far below 2^31), so nothing but the ABI
 * changes. An INTEGER argument outside the 32-bit range gives INFO = -(its
 * position), a descriptor entry -(100 * position + entry) -- the reference's
 * encoding of illegal arguments; routines without INFO return without work
 * (PDLANGE then returns 0). If libsl1x1gpu.so cannot be loaded beside this
 * library, INFO = -19999. IPIV: on input the entries IPIV(IA..IA+N-1) the
 * routine reads are narrowed, on output the entries it writes are widened;
 * the other entries are left untouched. IWORK: IWORK(1) (LIWMIN) is returned.
 * NUMROC is computed in 64-bit arithmetic directly.
 */
#ifndef SL1X1_ILP64_H
#define SL1X1_ILP64_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef long long sl_int64; /* Fortran INTEGER*8 */

void pdgetrf_(const sl_int64* M, const sl_int64* N, double* A, const sl_int64* IA,
              const sl_int64* JA, const sl_int64* DESCA, sl_int64* IPIV, sl_int64* INFO);
void pdgetrs_(const char* TRANS, const sl_int64* N, const sl_int64* NRHS, const double* A,
              const sl_int64* IA, const sl_int64* JA, const sl_int64* DESCA, const sl_int64* IPIV,
              double* B, const sl_int64* IB, const sl_int64* JB, const sl_int64* DESCB,
              sl_int64* INFO, size_t TRANS_len);
void pdgesv_(const sl_int64* N, const sl_int64* NRHS, double* A, const sl_int64* IA,
             const sl_int64* JA, const sl_int64* DESCA, sl_int64* IPIV, double* B,
             const sl_int64* IB, const sl_int64* JB, const sl_int64* DESCB, sl_int64* INFO);
double pdlange_(const char* NORM, const sl_int64* M, const sl_int64* N, const double* A,
                const sl_int64* IA, const sl_int64* JA, const sl_int64* DESCA, double* WORK,
                size_t NORM_len);
void pdgecon_(const char* NORM, const sl_int64* N, const double* A, const sl_int64* IA,
              const sl_int64* JA, const sl_int64* DESCA, const double* ANORM, double* RCOND,
              double* WORK, const sl_int64* LWORK, sl_int64* IWORK, const sl_int64* LIWORK,
              sl_int64* INFO, size_t NORM_len);
void pdgetri_(const sl_int64* N, double* A, const sl_int64* IA, const sl_int64* JA,
              const sl_int64* DESCA, const sl_int64* IPIV, double* WORK, const sl_int64* LWORK,
              sl_int64* IWORK, const sl_int64* LIWORK, sl_int64* INFO);
void pdgerfs_(const char* TRANS, const sl_int64* N, const sl_int64* NRHS, const double* A,
              const sl_int64* IA, const sl_int64* JA, const sl_int64* DESCA, const double* AF,
              const sl_int64* IAF, const sl_int64* JAF, const sl_int64* DESCAF,
              const sl_int64* IPIV, const double* B, const sl_int64* IB, const sl_int64* JB,
              const sl_int64* DESCB, double* X, const sl_int64* IX, const sl_int64* JX,
              const sl_int64* DESCX, double* FERR, double* BERR, double* WORK,
              const sl_int64* LWORK, sl_int64* IWORK, const sl_int64* LIWORK, sl_int64* INFO,
              size_t TRANS_len);
void pdgesvx_(const char* FACT, const char* TRANS, const sl_int64* N, const sl_int64* NRHS,
              double* A, const sl_int64* IA, const sl_int64* JA, const sl_int64* DESCA, double* AF,
              const sl_int64* IAF, const sl_int64* JAF, const sl_int64* DESCAF, sl_int64* IPIV,
              char* EQUED, double* R, double* C, double* B, const sl_int64* IB,
              const sl_int64* JB, const sl_int64* DESCB, double* X, const sl_int64* IX,
              const sl_int64* JX, const sl_int64* DESCX, double* RCOND, double* FERR, double* BERR,
              double* WORK, const sl_int64* LWORK, sl_int64* IWORK, const sl_int64* LIWORK,
              sl_int64* INFO, size_t FACT_len, size_t TRANS_len, size_t EQUED_len);
void pdgeequ_(const sl_int64* M, const sl_int64* N, const double* A, const sl_int64* IA,
              const sl_int64* JA, const sl_int64* DESCA, double* R, double* C, double* ROWCND,
              double* COLCND, double* AMAX, sl_int64* INFO);
void pdlaqge_(const sl_int64* M, const sl_int64* N, double* A, const sl_int64* IA,
              const sl_int64* JA, const sl_int64* DESCA, const double* R, const double* C,
              const double* ROWCND, const double* COLCND, const double* AMAX, char* EQUED,
              size_t EQUED_len);
void pdgemr2d_(const sl_int64* M, const sl_int64* N, const double* A, const sl_int64* IA,
               const sl_int64* JA, const sl_int64* DESCA, double* B, const sl_int64* IB,
               const sl_int64* JB, const sl_int64* DESCB, const sl_int64* ICTXT);
void descinit_(sl_int64* DESC, const sl_int64* M, const sl_int64* N, const sl_int64* MB,
               const sl_int64* NB, const sl_int64* IRSRC, const sl_int64* ICSRC,
               const sl_int64* ICTXT, const sl_int64* LLD, sl_int64* INFO);
sl_int64 numroc_(const sl_int64* N, const sl_int64* NB, const sl_int64* IPROC,
                 const sl_int64* ISRCPROC, const sl_int64* NPROCS);
void blacs_pinfo_(sl_int64* MYPNUM, sl_int64* NPROCS);
void blacs_get_(const sl_int64* ICTXT, const sl_int64* WHAT, sl_int64* VAL);
void blacs_gridinit_(sl_int64* ICTXT, const char* ORDER, const sl_int64* NPROW,
                     const sl_int64* NPCOL, size_t ORDER_len);
void blacs_gridinfo_(const sl_int64* ICTXT, sl_int64* NPROW, sl_int64* NPCOL, sl_int64* MYROW,
                     sl_int64* MYCOL);
void blacs_gridexit_(const sl_int64* ICTXT);
void blacs_exit_(const sl_int64* CONTINUE);

#ifdef __cplusplus
}
#endif

#endif /* SL1X1_ILP64_H */
