"""scalapack_gb300 -- GB300 (sm_103a) implementation of ScaLAPACK's dense LU
path on a 1x1 BLACS grid (PDGETRF / PDGETRS / PDGESV).

This module is the Python host-side mirror of the reference interface: the
functions below take the same arguments as the Fortran routines (M, N, A, IA,
JA, DESCA, IPIV, INFO ...) with numpy arrays in Fortran order standing in for
the Fortran arrays, and call the C ABI of ``libsl1x1gpu.so`` (declared in
``include/sl1x1.h``) through ctypes. There is no CPU implementation here: if the
CUDA library is missing the import of :func:`lib` raises, and without a GPU the
routines return INFO <= -10000.

Index and pivot conventions are the reference's: IA/JA/IB/JB are 1-based,
IPIV holds 1-based global row numbers (SRC/pdgetrf.f:118-121).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _build

__all__ = [
    "lib", "descinit", "numroc", "blacs_gridinit", "blacs_gridinfo", "blacs_gridexit",
    "blacs_exit", "pdgetrf", "pdgetrs", "pdgesv", "dgetrf_dev", "dgetrs_dev", "dgesv_dev",
    "DLEN", "CTXT_", "M_", "N_", "MB_", "NB_", "LLD_", "pdgerfs", "pdgesvx", "pdgeequ", "pdlaqge",
    "dgeequ_dev", "dgerfs_dev", "pdgemr2d",
]

DLEN = 9
DTYPE_, CTXT_, M_, N_, MB_, NB_, RSRC_, CSRC_, LLD_ = range(9)

_lib = None


def lib(build_if_missing: bool = False):
    """Load libsl1x1gpu.so (raises if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(
                f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            )
    L = C.CDLL(path)
    ip = C.POINTER(C.c_int)
    vp = C.c_void_p
    L.pdgetrf_.argtypes = [ip, ip, vp, ip, ip, ip, vp, ip]
    L.pdgetrf_.restype = None
    L.pdgetrs_.argtypes = [C.c_char_p, ip, ip, vp, ip, ip, ip, vp, vp, ip, ip, ip, ip, C.c_size_t]
    L.pdgetrs_.restype = None
    L.pdgesv_.argtypes = [ip, ip, vp, ip, ip, ip, vp, vp, ip, ip, ip, ip]
    L.pdgesv_.restype = None
    L.descinit_.argtypes = [vp, ip, ip, ip, ip, ip, ip, ip, ip, ip]
    L.descinit_.restype = None
    L.numroc_.argtypes = [ip, ip, ip, ip, ip]
    L.numroc_.restype = C.c_int
    L.blacs_pinfo_.argtypes = [ip, ip]
    L.blacs_get_.argtypes = [ip, ip, ip]
    L.blacs_gridinit_.argtypes = [ip, C.c_char_p, ip, ip, C.c_size_t]
    L.blacs_gridinfo_.argtypes = [ip, ip, ip, ip, ip]
    L.blacs_gridexit_.argtypes = [ip]
    L.blacs_exit_.argtypes = [ip]
    L.sl1x1_dgetrf_dev.argtypes = [C.c_int, C.c_int, vp, C.c_longlong, vp, C.c_int, vp]
    L.sl1x1_dgetrf_dev.restype = C.c_int
    L.sl1x1_dgetrs_dev.argtypes = [C.c_char, C.c_int, C.c_int, vp, C.c_longlong, vp, vp,
                                   C.c_longlong, vp]
    L.sl1x1_dgetrs_dev.restype = C.c_int
    L.sl1x1_dgesv_dev.argtypes = [C.c_int, C.c_int, vp, C.c_longlong, vp, vp, C.c_longlong,
                                  C.c_int, vp]
    L.sl1x1_dgesv_dev.restype = C.c_int
    L.sl1x1_dgetrf_noalloc.argtypes = [C.c_int, C.c_int, vp, C.c_longlong, vp, C.c_int, vp]
    L.sl1x1_dgetrf_noalloc.restype = C.c_int
    L.sl1x1_lowp_update_dev.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, vp, C.c_longlong, vp,
                                        C.c_longlong, vp, C.c_longlong, vp]
    L.sl1x1_lowp_update_dev.restype = C.c_int
    L.sl1x1_dgesv_ir_dev.argtypes = [C.c_int, C.c_int, vp, C.c_longlong, vp, vp, C.c_longlong, vp,
                                     C.c_longlong, C.c_int, C.c_int, C.c_double, C.c_int,
                                     C.POINTER(C.c_int), C.POINTER(C.c_double), vp]
    L.sl1x1_dgesv_ir_dev.restype = C.c_int
    L.sl1x1_batch_plan_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, vp, vp, vp, vp, vp, vp,
                                          vp, vp, C.c_int, C.c_double, C.c_int, vp]
    L.sl1x1_batch_plan_create.restype = C.c_int
    L.sl1x1_batch_plan_execute.argtypes = [vp, vp]
    L.sl1x1_batch_plan_execute.restype = C.c_int
    L.sl1x1_batch_plan_results.argtypes = [vp, vp, vp, vp, vp]
    L.sl1x1_batch_plan_results.restype = C.c_int
    L.sl1x1_batch_plan_shape.argtypes = [vp, vp, vp, vp]
    L.sl1x1_batch_plan_destroy.argtypes = [vp]
    L.pdlange_.argtypes = [C.c_char_p, ip, ip, vp, ip, ip, ip, vp, C.c_size_t]
    L.pdlange_.restype = C.c_double
    L.pdgecon_.argtypes = [C.c_char_p, ip, vp, ip, ip, ip, C.POINTER(C.c_double),
                           C.POINTER(C.c_double), vp, ip, vp, ip, ip, C.c_size_t]
    L.pdgecon_.restype = None
    L.pdgetri_.argtypes = [ip, vp, ip, ip, ip, vp, vp, ip, vp, ip, ip]
    L.pdgetri_.restype = None
    L.sl1x1_dlange_dev.argtypes = [C.c_char, C.c_int, C.c_int, vp, C.c_longlong, vp]
    L.sl1x1_dlange_dev.restype = C.c_double
    L.sl1x1_dgecon_dev.argtypes = [C.c_char, C.c_int, vp, C.c_longlong, C.c_double,
                                   C.POINTER(C.c_double), vp]
    L.sl1x1_dgecon_dev.restype = C.c_int
    L.sl1x1_dgetri_dev.argtypes = [C.c_int, vp, C.c_longlong, vp, vp]
    L.sl1x1_dgetri_dev.restype = C.c_int
    ip = C.POINTER(C.c_int)
    dp_ = C.POINTER(C.c_double)
    L.pdgerfs_.argtypes = [C.c_char_p, ip, ip, vp, ip, ip, ip, vp, ip, ip, ip, vp, vp, ip, ip, ip,
                           vp, ip, ip, ip, vp, vp, vp, ip, vp, ip, ip, C.c_size_t]
    L.pdgerfs_.restype = None
    L.pdgesvx_.argtypes = [C.c_char_p, C.c_char_p, ip, ip, vp, ip, ip, ip, vp, ip, ip, ip, vp,
                           C.c_char_p, vp, vp, vp, ip, ip, ip, vp, ip, ip, ip, dp_, vp, vp, vp, ip,
                           vp, ip, ip, C.c_size_t, C.c_size_t, C.c_size_t]
    L.pdgesvx_.restype = None
    L.pdgeequ_.argtypes = [ip, ip, vp, ip, ip, ip, vp, vp, dp_, dp_, dp_, ip]
    L.pdgeequ_.restype = None
    L.pdlaqge_.argtypes = [ip, ip, vp, ip, ip, ip, vp, vp, dp_, dp_, dp_, C.c_char_p, C.c_size_t]
    L.pdlaqge_.restype = None
    L.sl1x1_dgeequ_dev.argtypes = [C.c_int, C.c_int, vp, C.c_longlong, vp, vp, dp_, dp_, dp_, vp]
    L.sl1x1_dgeequ_dev.restype = C.c_int
    L.sl1x1_dgerfs_dev.argtypes = [C.c_char, C.c_int, C.c_int, vp, C.c_longlong, vp, C.c_longlong,
                                   vp, vp, C.c_longlong, vp, C.c_longlong, vp, vp, vp]
    L.sl1x1_dgerfs_dev.restype = C.c_int
    L.pdgemr2d_.argtypes = [ip, ip, vp, ip, ip, ip, vp, ip, ip, ip, ip]
    L.pdgemr2d_.restype = None
    L.sl1x1_finalize.argtypes = []
    L.sl1x1_set_default_nb.argtypes = [C.c_int]
    L.sl1x1_set_panel_rows.argtypes = [C.c_int]
    L.sl1x1_set_panel_ctas.argtypes = [C.c_int]
    L.sl1x1_set_panel_ib.argtypes = [C.c_int]
    L.sl1x1_set_panel_ib.restype = None
    L.sl1x1_set_panel_ctas.restype = None
    L.sl1x1_set_lowp_stages.argtypes = [C.c_int]
    L.sl1x1_set_f64_update.argtypes = [C.c_int]
    L.sl1x1_get_f64_update.restype = C.c_int
    L.sl1x1_set_ozgemm_tiles.argtypes = [C.c_int]
    L.sl1x1_ozgemm_dev.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, vp, C.c_longlong, vp,
                                   C.c_longlong, vp, C.c_longlong, vp]
    L.sl1x1_ozgemm_dev.restype = C.c_int
    L.sl1x1_ozgemm_fp64_routes.argtypes = []
    L.sl1x1_ozgemm_fp64_routes.restype = C.c_longlong
    L.sl1x1_set_lookahead.argtypes = [C.c_int]
    L.sl1x1_set_copy_chunks.argtypes = [C.c_int]
    L.sl1x1_debug_fail_alloc.argtypes = [C.c_int]
    L.sl1x1_debug_fail_alloc.restype = C.c_int
    L.sl1x1_debug_set_spin_limit.argtypes = [C.c_longlong]
    L.sl1x1_debug_set_spin_limit.restype = None
    L.sl1x1_set_ir_cost_ratio.argtypes = [C.c_double]
    L.sl1x1_set_ir_cost_ratio.restype = None
    L.sl1x1_set_update_reserve.argtypes = [C.c_int, C.c_int]
    L.sl1x1_set_split_step.argtypes = [C.c_int]
    L.sl1x1_set_update_share.argtypes = [C.c_double]
    L.sl1x1_set_inpanel_cap.argtypes = [C.c_int]
    L.sl1x1_set_inpanel_cap.restype = None
    L.sl1x1_set_update_share.restype = None
    L.sl1x1_set_split_step.restype = None
    L.sl1x1_set_update_reserve.restype = None
    L.sl1x1_device_ok.restype = C.c_int
    L.sl1x1_version.restype = C.c_char_p
    L.sl1x1_prof_enable.argtypes = [C.c_int]
    L.sl1x1_prof_read.argtypes = [C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.sl1x1_prof_read.restype = C.c_int
    L.sl1x1_launch_count.restype = C.c_longlong
    L.sl1x1_dmma_peak_tflops.restype = C.c_double
    _lib = L
    return L


def _i(v):
    return C.byref(C.c_int(int(v)))


def _arr(a, dtype):
    if a.dtype != dtype or not a.flags.f_contiguous:
        raise TypeError(f"expected a Fortran-ordered {dtype} array")
    return a.ctypes.data_as(C.c_void_p)


# ---------------------------------------------------------------- BLACS shim
def blacs_gridinit(nprow: int = 1, npcol: int = 1, order: str = "R") -> int:
    ctxt = C.c_int(0)
    lib().blacs_gridinit_(C.byref(ctxt), order.encode(), _i(nprow), _i(npcol), 1)
    return ctxt.value


def blacs_gridinfo(ictxt: int):
    v = [C.c_int() for _ in range(4)]
    lib().blacs_gridinfo_(_i(ictxt), *[C.byref(x) for x in v])
    return tuple(x.value for x in v)


def blacs_gridexit(ictxt: int):
    lib().blacs_gridexit_(_i(ictxt))


def blacs_exit(cont: int = 0):
    lib().blacs_exit_(_i(cont))


def numroc(n, nb, iproc, isrcproc, nprocs) -> int:
    return lib().numroc_(_i(n), _i(nb), _i(iproc), _i(isrcproc), _i(nprocs))


def descinit(m, n, mb, nb, irsrc, icsrc, ictxt, lld):
    """DESCINIT: returns (desc int32[9], info)."""
    desc = np.zeros(DLEN, dtype=np.int32)
    info = C.c_int()
    lib().descinit_(desc.ctypes.data_as(C.c_void_p), _i(m), _i(n), _i(mb), _i(nb), _i(irsrc),
                    _i(icsrc), _i(ictxt), _i(lld), C.byref(info))
    return desc, info.value


def _desc(desc):
    d = np.ascontiguousarray(desc, dtype=np.int32)
    return d, d.ctypes.data_as(C.POINTER(C.c_int))


# ---------------------------------------------------------------- LU routines
def pdgetrf(m, n, a, ia, ja, desca, ipiv) -> int:
    """PDGETRF(M, N, A, IA, JA, DESCA, IPIV, INFO): returns INFO; A and IPIV in place."""
    d, dp = _desc(desca)
    info = C.c_int()
    lib().pdgetrf_(_i(m), _i(n), _arr(a, np.float64), _i(ia), _i(ja), dp,
                   ipiv.ctypes.data_as(C.c_void_p), C.byref(info))
    return info.value


def pdgetrs(trans, n, nrhs, a, ia, ja, desca, ipiv, b, ib, jb, descb) -> int:
    """PDGETRS(TRANS, N, NRHS, A, IA, JA, DESCA, IPIV, B, IB, JB, DESCB, INFO)."""
    da, dap = _desc(desca)
    db, dbp = _desc(descb)
    info = C.c_int()
    lib().pdgetrs_(trans.encode()[:1], _i(n), _i(nrhs), _arr(a, np.float64), _i(ia), _i(ja), dap,
                   ipiv.ctypes.data_as(C.c_void_p), _arr(b, np.float64), _i(ib), _i(jb), dbp,
                   C.byref(info), 1)
    return info.value


def pdgesv(n, nrhs, a, ia, ja, desca, ipiv, b, ib, jb, descb) -> int:
    """PDGESV(N, NRHS, A, IA, JA, DESCA, IPIV, B, IB, JB, DESCB, INFO)."""
    da, dap = _desc(desca)
    db, dbp = _desc(descb)
    info = C.c_int()
    lib().pdgesv_(_i(n), _i(nrhs), _arr(a, np.float64), _i(ia), _i(ja), dap,
                  ipiv.ctypes.data_as(C.c_void_p), _arr(b, np.float64), _i(ib), _i(jb), dbp,
                  C.byref(info))
    return info.value


def pdlange(norm, m, n, a, ia, ja, desca) -> float:
    """PDLANGE(NORM, M, N, A, IA, JA, DESCA, WORK)."""
    d, dp = _desc(desca)
    work = np.zeros(max(1, m + n), dtype=np.float64)
    return lib().pdlange_(norm.encode()[:1], _i(m), _i(n), _arr(a, np.float64), _i(ia), _i(ja), dp,
                          work.ctypes.data_as(C.c_void_p), 1)


def pdgecon(norm, n, a, ia, ja, desca, anorm, lwork=None, liwork=None):
    """PDGECON: returns (rcond, info, work0, iwork0); lwork/liwork = -1 queries."""
    d, dp = _desc(desca)
    lw = 5 * n + 2 * max(1, int(desca[5])) + 16 if lwork is None else lwork
    liw = max(1, n) + 8 if liwork is None else liwork
    work = np.zeros(max(1, lw if lw > 0 else 1), dtype=np.float64)
    iwork = np.zeros(max(1, liw if liw > 0 else 1), dtype=np.int32)
    rc = C.c_double()
    info = C.c_int()
    lib().pdgecon_(norm.encode()[:1], _i(n), _arr(a, np.float64), _i(ia), _i(ja), dp,
                   C.byref(C.c_double(anorm)), C.byref(rc), work.ctypes.data_as(C.c_void_p), _i(lw),
                   iwork.ctypes.data_as(C.c_void_p), _i(liw), C.byref(info), 1)
    return rc.value, info.value, work[0], int(iwork[0])


def pdgetri(n, a, ia, ja, desca, ipiv, lwork=None, liwork=None):
    """PDGETRI: returns (info, work0, iwork0); A overwritten by inv(A)."""
    d, dp = _desc(desca)
    lw = max(1, (n + 64) * int(desca[5])) if lwork is None else lwork
    liw = int(desca[3]) + int(desca[5]) + 8 if liwork is None else liwork
    work = np.zeros(max(1, lw if lw > 0 else 1), dtype=np.float64)
    iwork = np.zeros(max(1, liw if liw > 0 else 1), dtype=np.int32)
    info = C.c_int()
    lib().pdgetri_(_i(n), _arr(a, np.float64), _i(ia), _i(ja), dp, ipiv.ctypes.data_as(C.c_void_p),
                   work.ctypes.data_as(C.c_void_p), _i(lw), iwork.ctypes.data_as(C.c_void_p), _i(liw),
                   C.byref(info))
    return info.value, work[0], int(iwork[0])


def _vec(a):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a contiguous float64 vector")
    return a.ctypes.data_as(C.c_void_p)


def pdgerfs(trans, n, nrhs, a, ia, ja, desca, af, iaf, jaf, descaf, ipiv, b, ib, jb, descb, x, ix,
            jx, descx, ferr, berr, lwork=None, liwork=None):
    """PDGERFS: X refined in place, FERR/BERR filled from JB; returns
    (info, work0, iwork0). lwork/liwork = -1 queries."""
    _, dpa = _desc(desca)
    _, dpf = _desc(descaf)
    _, dpb = _desc(descb)
    _, dpx = _desc(descx)
    lw = 3 * max(1, n) + 8 if lwork is None else lwork
    liw = max(1, n) + 8 if liwork is None else liwork
    work = np.zeros(max(1, lw if lw > 0 else 1), dtype=np.float64)
    iwork = np.zeros(max(1, liw if liw > 0 else 1), dtype=np.int32)
    info = C.c_int()
    lib().pdgerfs_(trans.encode()[:1], _i(n), _i(nrhs), _arr(a, np.float64), _i(ia), _i(ja), dpa,
                   _arr(af, np.float64), _i(iaf), _i(jaf), dpf, ipiv.ctypes.data_as(C.c_void_p),
                   _arr(b, np.float64), _i(ib), _i(jb), dpb, _arr(x, np.float64), _i(ix), _i(jx), dpx,
                   _vec(ferr), _vec(berr), work.ctypes.data_as(C.c_void_p), _i(lw),
                   iwork.ctypes.data_as(C.c_void_p), _i(liw), C.byref(info), 1)
    return info.value, work[0], int(iwork[0])


def pdgesvx(fact, trans, n, nrhs, a, ia, ja, desca, af, iaf, jaf, descaf, ipiv, equed, r, c, b, ib,
            jb, descb, x, ix, jx, descx, ferr, berr, lwork=None, liwork=None):
    """PDGESVX: returns dict(info, equed, rcond, work0, iwork0); A, AF, IPIV,
    R, C, B, X, FERR and BERR are updated in place as the reference does."""
    _, dpa = _desc(desca)
    _, dpf = _desc(descaf)
    _, dpb = _desc(descb)
    _, dpx = _desc(descx)
    nb = max(1, int(desca[5]))
    lw = 6 * max(1, n) + 4 * nb + 64 if lwork is None else lwork
    liw = max(1, n) + 8 if liwork is None else liwork
    work = np.zeros(max(1, lw if lw > 0 else 1), dtype=np.float64)
    iwork = np.zeros(max(1, liw if liw > 0 else 1), dtype=np.int32)
    info = C.c_int()
    rcond = C.c_double(-1.0)
    eq = C.create_string_buffer(equed.encode()[:1], 2)
    lib().pdgesvx_(fact.encode()[:1], trans.encode()[:1], _i(n), _i(nrhs), _arr(a, np.float64),
                   _i(ia), _i(ja), dpa, _arr(af, np.float64), _i(iaf), _i(jaf), dpf,
                   ipiv.ctypes.data_as(C.c_void_p), eq, _vec(r), _vec(c), _arr(b, np.float64), _i(ib),
                   _i(jb), dpb, _arr(x, np.float64), _i(ix), _i(jx), dpx, C.byref(rcond), _vec(ferr),
                   _vec(berr), work.ctypes.data_as(C.c_void_p), _i(lw),
                   iwork.ctypes.data_as(C.c_void_p), _i(liw), C.byref(info), 1, 1, 1)
    return dict(info=info.value, equed=eq.value.decode(), rcond=rcond.value, work0=work[0],
                iwork0=int(iwork[0]))


def pdgemr2d(m, n, a, ia, ja, desca, b, ib, jb, descb, ictxt=-1):
    """PDGEMR2D between this process's 1x1 contexts: sub(A) copied into sub(B)."""
    _, dpa = _desc(desca)
    _, dpb = _desc(descb)
    lib().pdgemr2d_(_i(m), _i(n), _arr(a, np.float64), _i(ia), _i(ja), dpa, _arr(b, np.float64),
                    _i(ib), _i(jb), dpb, _i(ictxt))


def pdgeequ(m, n, a, ia, ja, desca, r, c):
    """PDGEEQU: R(IA..) and C(JA..) filled; returns (info, rowcnd, colcnd, amax)."""
    _, dp = _desc(desca)
    rc, cc, am = C.c_double(-1.0), C.c_double(-1.0), C.c_double(-1.0)
    info = C.c_int()
    lib().pdgeequ_(_i(m), _i(n), _arr(a, np.float64), _i(ia), _i(ja), dp, _vec(r), _vec(c),
                   C.byref(rc), C.byref(cc), C.byref(am), C.byref(info))
    return info.value, rc.value, cc.value, am.value


def pdlaqge(m, n, a, ia, ja, desca, r, c, rowcnd, colcnd, amax) -> str:
    """PDLAQGE: sub(A) scaled in place; returns EQUED."""
    _, dp = _desc(desca)
    eq = C.create_string_buffer(b"?", 2)
    lib().pdlaqge_(_i(m), _i(n), _arr(a, np.float64), _i(ia), _i(ja), dp, _vec(r), _vec(c),
                   C.byref(C.c_double(rowcnd)), C.byref(C.c_double(colcnd)),
                   C.byref(C.c_double(amax)), eq, 1)
    return eq.value.decode()


# ------------------------------------------------------------ phase timers
PHASES = ["panel", "laswp", "trsm", "gemm", "solve", "mixed_gemm", "mixed_panel", "refine",
          "batched", "residual", "precond", "panel_kernel", "panel_update", "panel_inverse"]


def prof_enable(on: bool = True):
    lib().sl1x1_prof_enable(1 if on else 0)


def prof_read():
    """{phase: (launches, device ms, algorithmic flops, algorithmic bytes)}."""
    out = {}
    for i, name in enumerate(PHASES):
        n, ms, fl, by = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        lib().sl1x1_prof_read(i, C.byref(n), C.byref(ms), C.byref(fl), C.byref(by))
        out[name] = (n.value, ms.value, fl.value, by.value)
    return out


def launch_count() -> int:
    return int(lib().sl1x1_launch_count())


# ------------------------------------------------------- device entry points
def _stream_ptr(stream):
    if stream is None:
        return None
    return C.c_void_p(int(stream))


def dgetrf_dev(m, n, a_ptr, ldda, ipiv_ptr, nb=0, stream=None) -> int:
    """sl1x1_dgetrf_dev on device pointers (e.g. torch ``.data_ptr()``)."""
    return lib().sl1x1_dgetrf_dev(m, n, C.c_void_p(a_ptr), ldda, C.c_void_p(ipiv_ptr), nb,
                                  _stream_ptr(stream))


def set_f64_update(mode: int):
    """Trailing-update arithmetic of the FP64 factorization: 1 = sliced BF16
    tensor-core product (default), 0 = FP64 DMMA."""
    lib().sl1x1_set_f64_update(int(mode))


def get_f64_update() -> int:
    return int(lib().sl1x1_get_f64_update())


def ozgemm_dev(m, n, k, alpha, a_ptr, ldda, b_ptr, lddb, c_ptr, lddc, stream=None) -> int:
    """C += alpha * A * B (FP64 device arrays) through the sliced tensor-core product."""
    return lib().sl1x1_ozgemm_dev(m, n, k, float(alpha), C.c_void_p(a_ptr), ldda, C.c_void_p(b_ptr),
                                  lddb, C.c_void_p(c_ptr), lddc, _stream_ptr(stream))


def dgetrf_noalloc(m, n, a_ptr, ldda, ipiv_ptr, nb=0, stream=None) -> int:
    """sl1x1_dgetrf_noalloc: the factorization without any GPU allocation."""
    return lib().sl1x1_dgetrf_noalloc(m, n, C.c_void_p(a_ptr), ldda, C.c_void_p(ipiv_ptr), nb,
                                      _stream_ptr(stream))


IR_STATS = ["classical", "gmres_outer", "gmres_inner", "fell_back", "sresid", "anorm",
            "factor_ms", "refine_ms"]


def dgesv_ir_dev(n, nrhs, a_ptr, ldda, ipiv_ptr, b_ptr, lddb, x_ptr, lddx, fmt="bf16", nb=256,
                 tol=1.0, keep_a=True, stream=None):
    """Mixed-precision LU-IR (sl1x1_dgesv_ir_dev). Returns (info, iter, stats dict)."""
    it = C.c_int()
    st = (C.c_double * 8)()
    f = {"bf16": 0, "fp16": 1, "bf16x3": 2}[fmt] if isinstance(fmt, str) else int(fmt)
    info = lib().sl1x1_dgesv_ir_dev(n, nrhs, C.c_void_p(a_ptr), ldda, C.c_void_p(ipiv_ptr),
                                    C.c_void_p(b_ptr), lddb, C.c_void_p(x_ptr), lddx, f, nb,
                                    float(tol), 1 if keep_a else 0, C.byref(it), st,
                                    _stream_ptr(stream))
    return info, it.value, dict(zip(IR_STATS, list(st)))


class BatchPlan:
    """Batched solver plan over device arrays (torch tensors or raw pointers).

    systems: list of (a_ptr, lda, n, b_ptr, ldb, nrhs, x_ptr, ldx); mode 0 = FP64,
    1 = FP32 factors + FP64 refinement. execute() replays the captured CUDA graph.
    """

    def __init__(self, systems, mode=0, tol=1.0, autotune=True, stream=None):
        k = len(systems)
        I = C.c_int * k
        P = C.c_void_p * k
        self.batch = k
        self._keep = (I(*[s[2] for s in systems]), I(*[s[5] for s in systems]),
                      P(*[s[0] for s in systems]), I(*[s[1] for s in systems]),
                      P(*[s[3] for s in systems]), I(*[s[4] for s in systems]),
                      P(*[s[6] for s in systems]), I(*[s[7] for s in systems]))
        n, r, a, lda, b, ldb, x, ldx = self._keep
        self.plan = C.c_void_p()
        info = lib().sl1x1_batch_plan_create(C.byref(self.plan), C.c_int(k), n, r, a, lda, b, ldb,
                                             x, ldx, C.c_int(mode), C.c_double(float(tol)),
                                             C.c_int(1 if autotune else 0), _stream_ptr(stream))
        if info != 0:
            raise RuntimeError(f"sl1x1_batch_plan_create INFO={info}")
        self.stream = stream

    def execute(self):
        info = lib().sl1x1_batch_plan_execute(self.plan, _stream_ptr(self.stream))
        if info != 0:
            raise RuntimeError(f"sl1x1_batch_plan_execute INFO={info}")

    def results(self):
        info = (C.c_int * self.batch)()
        its = (C.c_int * self.batch)()
        sr = (C.c_double * self.batch)()
        lib().sl1x1_batch_plan_results(self.plan, info, its, sr, _stream_ptr(self.stream))
        return list(info), list(its), list(sr)

    def shape(self):
        t, c, s = C.c_int(), C.c_int(), C.c_int()
        lib().sl1x1_batch_plan_shape(self.plan, C.byref(t), C.byref(c), C.byref(s))
        return {"threads": t.value, "chunk": c.value, "ctas_per_sm": s.value}

    def close(self):
        if self.plan:
            lib().sl1x1_batch_plan_destroy(self.plan)
            self.plan = C.c_void_p()


def dgetrs_dev(trans, n, nrhs, a_ptr, ldda, ipiv_ptr, b_ptr, lddb, stream=None) -> int:
    return lib().sl1x1_dgetrs_dev(trans.encode()[:1], n, nrhs, C.c_void_p(a_ptr), ldda,
                                  C.c_void_p(ipiv_ptr), C.c_void_p(b_ptr), lddb,
                                  _stream_ptr(stream))


def dgeequ_dev(m, n, a_ptr, ldda, r_ptr, c_ptr, stream=None):
    """PDGEEQU on device data: returns (info, rowcnd, colcnd, amax)."""
    rc, cc, am = C.c_double(-1.0), C.c_double(-1.0), C.c_double(-1.0)
    info = lib().sl1x1_dgeequ_dev(m, n, a_ptr, ldda, r_ptr, c_ptr, C.byref(rc), C.byref(cc),
                                  C.byref(am), _stream_ptr(stream))
    return info, rc.value, cc.value, am.value


def dgerfs_dev(trans, n, nrhs, a_ptr, ldda, af_ptr, lddaf, ipiv_ptr, b_ptr, lddb, x_ptr, lddx,
               stream=None):
    """PDGERFS on device data (ipiv 1-based): returns (info, ferr, berr)."""
    ferr = np.zeros(max(1, nrhs))
    berr = np.zeros(max(1, nrhs))
    info = lib().sl1x1_dgerfs_dev(trans.encode()[:1], n, nrhs, a_ptr, ldda, af_ptr, lddaf, ipiv_ptr,
                                  b_ptr, lddb, x_ptr, lddx, ferr.ctypes.data_as(C.c_void_p),
                                  berr.ctypes.data_as(C.c_void_p), _stream_ptr(stream))
    return info, ferr[:nrhs], berr[:nrhs]


def dgesv_dev(n, nrhs, a_ptr, ldda, ipiv_ptr, b_ptr, lddb, nb=0, stream=None) -> int:
    return lib().sl1x1_dgesv_dev(n, nrhs, C.c_void_p(a_ptr), ldda, C.c_void_p(ipiv_ptr),
                                 C.c_void_p(b_ptr), lddb, nb, _stream_ptr(stream))
