"""ctypes front end of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

The oracle is a C restatement of ScaLAPACK's 1x1-grid LU path
(SRC/pdgetrf.f, SRC/pdgetf2.f, SRC/pdlaswp.f, SRC/pdgetrs.f, SRC/pdlapv2.f,
PBLAS/SRC/PTOOLS/PB_CptrsmAB.c, PB_CpgemmAB.c) plus the LU tester's generator
(TESTING/traditional/LIN/pdmatgen.f, pmatgeninc.f) and residual checks
(LIN/pdlaschk.f, LIN/pdlafchk.f).  Only tests, the smoke check and the
benchmark's CPU-baseline leg import this module; the product library never
does.

Arrays are numpy float64 in Fortran (column-major) order; pivots are int32,
1-based, as the reference stores them.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "sl_oracle.c")
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "libsl_oracle.so")

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with gcc into oracle/_build/ (recipe: oracle/Makefile)."""
    os.makedirs(_BUILD, exist_ok=True)
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < os.path.getmtime(_SRC):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def find_host_blas():
    """Locate the host OpenBLAS that scipy bundles (LP64, 'scipy_' prefix)."""
    try:
        import scipy  # noqa: F401

        base = os.path.dirname(os.path.dirname(sys.modules["scipy"].__file__))
    except Exception:  # pragma: no cover - scipy is present in both environments
        return None, None
    cands = sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
    cands = [c for c in cands if "64_" not in os.path.basename(c)]
    if cands:
        return cands[0], "scipy_"
    return None, None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    build()
    L = C.CDLL(_SO)
    dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
    L.orc_load_blas.argtypes = [C.c_char_p, C.c_char_p]
    L.orc_load_blas.restype = C.c_int
    L.orc_blas_loaded.restype = C.c_int
    L.orc_set_threads.argtypes = [C.c_int]
    L.orc_lcg_state.argtypes = [C.c_int, C.c_uint64]
    L.orc_lcg_state.restype = C.c_uint32
    L.orc_matgen.argtypes = [C.c_int] * 9 + [C.c_void_p, C.c_int]
    L.orc_pdgetrf.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                              C.c_int, C.c_void_p]
    L.orc_pdgetrf.restype = C.c_int
    L.orc_pdgetrs.argtypes = [C.c_char, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                              C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
    L.orc_lapack_dgetrf.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    L.orc_lapack_dgetrf.restype = C.c_int
    L.orc_lapack_dgetrs.argtypes = [C.c_char, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                    C.c_void_p, C.c_int]
    L.orc_lapack_dgetrs.restype = C.c_int
    L.orc_dgemm.argtypes = [C.c_char, C.c_char, C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p,
                            C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_int]
    L.orc_norm_inf.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int]
    L.orc_norm_inf.restype = C.c_double
    L.orc_sresid.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                             C.c_int, C.c_double]
    L.orc_sresid.restype = C.c_double
    L.orc_fresid.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                             C.c_double]
    L.orc_fresid.restype = C.c_double
    L.orc_eps.restype = C.c_double
    L.orc_set_recorder.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
    L.orc_gen_conditioned.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_int]
    L.orc_pdgeequ.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.orc_pdgeequ.restype = C.c_int
    L.orc_pdlaqge.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                              C.c_void_p, C.c_double, C.c_double, C.c_double]
    L.orc_pdlaqge.restype = C.c_char
    L.orc_pdlange.argtypes = [C.c_char, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int]
    L.orc_pdlange.restype = C.c_double
    L.orc_pdgecon.argtypes = [C.c_char, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double]
    L.orc_pdgecon.restype = C.c_double
    L.orc_pdgetri.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
    L.orc_pdgetri.restype = C.c_int
    L.orc_pdgerfs.argtypes = [C.c_char, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                              C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                              C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int,
                              C.c_void_p, C.c_void_p]
    L.orc_pdgerfs.restype = None
    L.orc_pdgesvx.argtypes = [C.c_char, C.c_char, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int,
                              C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                              C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                              C.c_void_p, C.c_void_p]
    L.orc_pdgesvx.restype = C.c_int
    path, prefix = find_host_blas()
    if path:
        L.orc_load_blas(path.encode(), prefix.encode())
    _lib = L
    del dp, ip
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def blas_loaded() -> bool:
    return bool(lib().orc_blas_loaded())


def use_fallback_blas():
    lib().orc_use_fallback_blas()


def reload_host_blas():
    path, prefix = find_host_blas()
    if path:
        return lib().orc_load_blas(path.encode(), prefix.encode()) == 0
    return False


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def lcg_state(seed: int, steps: int) -> int:
    return int(lib().orc_lcg_state(seed, steps))


def matgen(M, N, seed, kind=0, diag=False, i0=0, j0=0, nrows=None, ncols=None, ld=None):
    """Block (i0:i0+nrows, j0:j0+ncols) of PDMATGEN's M x N matrix on a 1x1 grid.

    kind 0: tester values 1-2*PDRAND on (-1,1]; kind 1: 0.5-PDRAND on (-0.5,0.5].
    """
    nrows = M - i0 if nrows is None else nrows
    ncols = N - j0 if ncols is None else ncols
    ld = max(1, nrows) if ld is None else ld
    out = np.zeros((ld, max(ncols, 0)), dtype=np.float64, order="F")
    lib().orc_matgen(M, N, seed, kind, 1 if diag else 0, i0, j0, nrows, ncols, _p(out), ld)
    return out


def pdgetrf(m, n, A, ia=1, ja=1, nb=64, mglob=None, ipiv=None):
    """Factor sub(A) in place (A: Fortran-ordered local array). Returns (ipiv, info)."""
    assert A.dtype == np.float64 and A.flags.f_contiguous
    lda = A.shape[0]
    mglob = A.shape[0] if mglob is None else mglob
    if ipiv is None:
        ipiv = np.zeros(A.shape[0] + nb, dtype=np.int32)
    info = lib().orc_pdgetrf(m, n, _p(A), lda, ia, ja, nb, mglob, _p(ipiv))
    return ipiv, info


def pdgetrs(trans, n, nrhs, A, ipiv, B, ia=1, ja=1, ib=1, jb=1):
    assert B.dtype == np.float64 and B.flags.f_contiguous
    lib().orc_pdgetrs(trans.encode()[:1], n, nrhs, _p(A), A.shape[0], ia, ja, _p(ipiv), _p(B),
                      B.shape[0], ib, jb)


def lapack_dgetrf(A):
    A = np.asfortranarray(A.copy())
    m, n = A.shape
    ipiv = np.zeros(min(m, n), dtype=np.int32)
    info = lib().orc_lapack_dgetrf(m, n, _p(A), m, _p(ipiv))
    return A, ipiv, info


def lapack_dgesv(A, B):
    """Host LAPACK dgetrf + dgetrs (the BLAS library's own LU, not the
    restatement), in place on Fortran-ordered A and B. Returns (ipiv, info)."""
    assert A.flags.f_contiguous and B.flags.f_contiguous
    n = A.shape[0]
    ipiv = np.zeros(n, dtype=np.int32)
    info = lib().orc_lapack_dgetrf(n, n, _p(A), A.shape[0], _p(ipiv))
    if info == 0:
        lib().orc_lapack_dgetrs(b"N", n, B.shape[1], _p(A), A.shape[0], _p(ipiv), _p(B), B.shape[0])
    return ipiv, info


def dgemm(ta, tb, alpha, a, b, beta, c):
    m = c.shape[0]
    n = c.shape[1]
    k = a.shape[1] if ta == "N" else a.shape[0]
    lib().orc_dgemm(ta.encode(), tb.encode(), m, n, k, alpha, _p(a), a.shape[0], _p(b), b.shape[0],
                    beta, _p(c), c.shape[0])


def norm_inf(X):
    X = np.asfortranarray(X)
    return lib().orc_norm_inf(X.shape[0], X.shape[1], _p(X), X.shape[0])


def eps():
    return lib().orc_eps()


def sresid(A0, B0, X):
    A0 = np.asfortranarray(A0); B0 = np.asfortranarray(B0); X = np.asfortranarray(X)
    n = A0.shape[0]
    nrhs = B0.shape[1]
    anorm = norm_inf(A0)
    return lib().orc_sresid(n, nrhs, _p(A0), A0.shape[0], _p(B0), B0.shape[0], _p(X), X.shape[0],
                            anorm)


def fresid(LU, ipiv_rel, A0):
    LU = np.asfortranarray(LU); A0 = np.asfortranarray(A0)
    ipiv_rel = np.ascontiguousarray(ipiv_rel, dtype=np.int32)
    m, n = A0.shape
    return lib().orc_fresid(m, n, _p(LU), LU.shape[0], _p(ipiv_rel), _p(A0), A0.shape[0],
                            norm_inf(A0))


class Recorder:
    """Near-tie recorder (top-2 |candidates| per column) with optional forced pivots."""

    def __init__(self, ncols, force=None):
        self.top1 = np.full(ncols, -1.0)
        self.top2 = np.full(ncols, -1.0)
        self.force = None if force is None else np.ascontiguousarray(force, dtype=np.int32)
        self.ncols = ncols

    def __enter__(self):
        lib().orc_set_recorder(_p(self.top1), _p(self.top2), self.ncols,
                               None if self.force is None else _p(self.force))
        return self

    def __exit__(self, *exc):
        lib().orc_set_recorder(None, None, 0, None)

    def near_ties(self, rel=1e-10):
        """Columns whose two largest candidates differ by less than `rel` relative."""
        t1, t2 = self.top1, self.top2
        ok = (t1 > 0) & (t2 >= 0)
        gap = np.where(ok, (t1 - t2) / np.where(t1 > 0, t1, 1.0), np.inf)
        return np.nonzero(gap < rel)[0]


def gen_conditioned(n, kappa, nrefl=64, seed=1000):
    A = np.zeros((n, n), dtype=np.float64, order="F")
    lib().orc_gen_conditioned(n, nrefl, float(kappa), seed, _p(A), n)
    return A


def solve_reference(A, B, nb=64):
    """Oracle PDGESV on a 1x1 grid: returns (LU, ipiv(1-based rel), X, info)."""
    n = A.shape[0]
    LU = np.asfortranarray(A.copy())
    ipiv, info = pdgetrf(n, n, LU, nb=nb)
    X = np.asfortranarray(B.copy())
    if info == 0:
        pdgetrs("N", n, B.shape[1], LU, ipiv, X)
    return LU, ipiv[:n].copy(), X, info


# ---- expert driver (PDGEEQU / PDLAQGE / PDLANGE / PDGECON / PDGERFS / PDGESVX) ----

def pdgeequ(A):
    """PDGEEQU of a Fortran-order matrix: (R, C, rowcnd, colcnd, amax, info)."""
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    R = np.zeros(max(m, 1))
    Cv = np.zeros(max(n, 1))
    out = (C.c_double * 3)()
    info = lib().orc_pdgeequ(m, n, _p(A), max(m, 1), 1, 1, _p(R), _p(Cv), C.byref(out, 0),
                             C.byref(out, 8), C.byref(out, 16))
    return R[:m], Cv[:n], out[0], out[1], out[2], info


def pdlaqge(A, R, Cv, rowcnd, colcnd, amax):
    """PDLAQGE: (scaled copy of A, EQUED)."""
    A = np.array(A, dtype=np.float64, order="F")
    m, n = A.shape
    R = np.ascontiguousarray(R, dtype=np.float64)
    Cv = np.ascontiguousarray(Cv, dtype=np.float64)
    eq = lib().orc_pdlaqge(m, n, _p(A), max(m, 1), 1, 1, _p(R), _p(Cv), rowcnd, colcnd, amax)
    return A, eq.decode()


def pdlange(norm, A):
    A = np.asfortranarray(A, dtype=np.float64)
    return lib().orc_pdlange(norm.encode(), A.shape[0], _p(A), max(A.shape[0], 1), 1, 1)


def pdgecon(norm, LU, anorm):
    LU = np.asfortranarray(LU, dtype=np.float64)
    return lib().orc_pdgecon(norm.encode(), LU.shape[0], _p(LU), max(LU.shape[0], 1), 1, 1, anorm)


def pdgetri(LU, ipiv_rel, nb=64):
    """PDGETRI on a 1x1 grid from the factors L, U and 0-based relative pivots (as
    pdgetrf leaves them, minus one): (INFO, inv(A) or the unchanged LU)."""
    X = np.asfortranarray(np.array(LU, dtype=np.float64))
    piv = np.ascontiguousarray(ipiv_rel, dtype=np.int32)
    n = X.shape[0]
    info = lib().orc_pdgetri(n, _p(X), max(n, 1), 1, 1, _p(piv), nb)
    return info, X


def pdgerfs(trans, A, AF, ipiv, B, X):
    """PDGERFS with IA = IAF = IB = IX = 1: (refined X, FERR, BERR); ipiv holds
    global 1-based rows as PDGETRF writes them."""
    A = np.asfortranarray(A, dtype=np.float64)
    AF = np.asfortranarray(AF, dtype=np.float64)
    B = np.asfortranarray(B, dtype=np.float64)
    X = np.array(X, dtype=np.float64, order="F")
    n, nrhs = B.shape
    ip = np.ascontiguousarray(ipiv, dtype=np.int32)
    ferr = np.zeros(max(nrhs, 1))
    berr = np.zeros(max(nrhs, 1))
    ld = max(n, 1)
    lib().orc_pdgerfs(trans.encode(), n, nrhs, _p(A), ld, 1, 1, _p(AF), ld, 1, 1, _p(ip), _p(B), ld,
                      1, 1, _p(X), ld, 1, 1, _p(ferr), _p(berr))
    return X, ferr[:nrhs], berr[:nrhs]


def pdgesvx(fact, trans, A, B, AF=None, ipiv=None, equed="N", R=None, Cv=None, nb=64):
    """PDGESVX with IA = IAF = IB = IX = 1 on copies of the inputs; returns a
    dict of every output (A and B as modified by equilibration)."""
    A = np.array(A, dtype=np.float64, order="F")
    B = np.array(B, dtype=np.float64, order="F")
    n, nrhs = B.shape
    ld = max(n, 1)
    AF = np.zeros((n, n), order="F") if AF is None else np.array(AF, dtype=np.float64, order="F")
    ip = np.zeros(max(n, 1), np.int32) if ipiv is None else np.array(ipiv, dtype=np.int32)
    R = np.zeros(max(n, 1)) if R is None else np.array(R, dtype=np.float64)
    Cv = np.zeros(max(n, 1)) if Cv is None else np.array(Cv, dtype=np.float64)
    X = np.zeros((n, nrhs), order="F")
    eq = C.create_string_buffer(equed.encode(), 2)
    rcond = C.c_double(0.0)
    ferr = np.zeros(max(nrhs, 1))
    berr = np.zeros(max(nrhs, 1))
    info = lib().orc_pdgesvx(fact.encode(), trans.encode(), n, nrhs, _p(A), ld, 1, 1, _p(AF), ld, 1,
                             1, n, nb, _p(ip), eq, _p(R), _p(Cv), _p(B), ld, 1, 1, _p(X), ld, 1, 1,
                             C.byref(rcond), _p(ferr), _p(berr))
    return dict(info=info, A=A, AF=AF, ipiv=ip[:n], equed=eq.value.decode(), R=R[:n], C=Cv[:n],
                B=B, X=X, rcond=rcond.value, ferr=ferr[:nrhs], berr=berr[:nrhs])
