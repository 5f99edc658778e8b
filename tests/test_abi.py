"""CPU tests of the C ABI: the library loads, exports every declared symbol,
and the host logic (BLACS shim, DESCINIT/NUMROC, argument validation with the
reference's INFO codes) behaves like the reference. None of these calls reach
the GPU: argument errors are detected before any device work.
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sl1x1.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:void|int|const char\s*\*)\s*(\w+)\s*\(", txt, flags=re.M)))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for must in ("pdgetrf_", "pdgetrs_", "pdgesv_", "descinit_", "numroc_", "blacs_gridinit_",
                 "blacs_gridinfo_", "sl1x1_dgetrf_dev"):
        assert must in names


def test_library_exports_every_declared_symbol(sl):
    L = sl.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", sl._build.lib_path()], capture_output=True,
                         text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    assert set(declared_functions()) <= exported


def test_version_string(sl):
    assert b"sm_103a" in sl.lib().sl1x1_version()


def test_blacs_shim_contexts(sl):
    ctxt = sl.blacs_gridinit(1, 1)
    assert sl.blacs_gridinfo(ctxt) == (1, 1, 0, 0)
    bad = sl.blacs_gridinit(2, 2)
    assert sl.blacs_gridinfo(bad) == (-1, -1, -1, -1)
    sl.blacs_gridexit(ctxt)
    assert sl.blacs_gridinfo(ctxt) == (-1, -1, -1, -1)
    me, np_ = C.c_int(), C.c_int()
    sl.lib().blacs_pinfo_(C.byref(me), C.byref(np_))
    assert (me.value, np_.value) == (0, 1)


def _numroc_ref(n, nb, iproc, isrc, nprocs):
    # TOOLS/numroc.f:53-76
    mydist = (nprocs + iproc - isrc) % nprocs
    nblocks = n // nb
    r = (nblocks // nprocs) * nb
    extra = nblocks % nprocs
    if mydist < extra:
        r += nb
    elif mydist == extra:
        r += n % nb
    return r


@pytest.mark.parametrize("n,nb,ip,isrc,npr", [(10, 3, 0, 0, 1), (17, 4, 1, 0, 3), (100, 7, 2, 1, 4),
                                              (0, 5, 0, 0, 2), (65, 64, 1, 0, 2)])
def test_numroc(sl, n, nb, ip, isrc, npr):
    assert sl.numroc(n, nb, ip, isrc, npr) == _numroc_ref(n, nb, ip, isrc, npr)


def test_descinit(sl):
    ctxt = sl.blacs_gridinit(1, 1)
    d, info = sl.descinit(100, 50, 32, 32, 0, 0, ctxt, 128)
    assert info == 0
    assert list(d) == [1, ctxt, 100, 50, 32, 32, 0, 0, 128]
    d, info = sl.descinit(100, 50, 32, 32, 0, 0, ctxt, 10)  # LLD < M
    assert info == -9 and d[8] == 100
    d, info = sl.descinit(-1, 50, 32, 32, 0, 0, ctxt, 128)
    assert info == -2


@pytest.fixture()
def ctx(sl):
    return sl.blacs_gridinit(1, 1)


def _getrf_info(sl, m, n, ia, ja, desc):
    a = np.zeros((max(desc[8], 1), max(desc[3], 1)), dtype=np.float64, order="F")
    ipiv = np.zeros(max(desc[2], 1) + max(desc[4], 1), dtype=np.int32)
    return sl.pdgetrf(m, n, a, ia, ja, desc, ipiv)


def _desc(ctx, m=8, n=8, mb=4, nb=4, lld=8, dtype=1, rsrc=0, csrc=0):
    return np.array([dtype, ctx, m, n, mb, nb, rsrc, csrc, lld], dtype=np.int32)


# (M, N, IA, JA, descriptor changes) -> INFO, derived from SRC/pdgetrf.f:170-197
# and TOOLS/chk1mat.f (array arguments: -(position*100 + entry); DESCA is
# argument 6, IA is 4, JA is 5, M is 1, N is 2).
GETRF_CASES = [
    (dict(), 8, 8, 1, 1, 0, "ok"),
    (dict(dtype=2), 8, 8, 1, 1, -601, "DTYPE"),
    (dict(), -1, 8, 1, 1, -1, "M<0"),
    (dict(), 8, -1, 1, 1, -2, "N<0"),
    (dict(), 8, 8, 0, 1, -4, "IA<1"),
    (dict(), 8, 8, 1, 0, -5, "JA<1"),
    (dict(mb=0), 8, 8, 1, 1, -605, "MB<1"),
    (dict(nb=0), 8, 8, 1, 1, -606, "NB<1"),
    (dict(rsrc=1), 8, 8, 1, 1, -607, "RSRC"),
    (dict(csrc=1), 8, 8, 1, 1, -608, "CSRC"),
    (dict(lld=4), 8, 8, 1, 1, -609, "LLD<M_"),
    (dict(m=0), 8, 8, 1, 1, -603, "M_<1"),
    (dict(n=0), 8, 8, 1, 1, -604, "N_<1"),
    (dict(), 8, 8, 9, 1, -4, "IA>M_"),
    (dict(), 8, 8, 1, 9, -5, "JA>N_"),
    (dict(), 8, 8, 2, 1, -1, "IA+M-1>M_"),
    (dict(), 4, 8, 1, 2, -2, "JA+N-1>N_"),
    (dict(), 4, 4, 2, 1, -4, "IA misaligned"),
    (dict(), 4, 4, 1, 2, -5, "JA misaligned"),
    (dict(nb=2), 4, 4, 1, 1, -606, "MB != NB"),
]


@pytest.mark.parametrize("chg,m,n,ia,ja,expect,why", GETRF_CASES, ids=[c[-1] for c in GETRF_CASES])
def test_pdgetrf_argument_errors(sl, ctx, capfd, chg, m, n, ia, ja, expect, why):
    if expect == 0:
        pytest.skip("valid arguments reach the GPU")
    d = _desc(ctx, **chg)
    info = _getrf_info(sl, m, n, ia, ja, d)
    assert info == expect, why
    out = capfd.readouterr().out
    assert f"On entry to PDGETRF parameter number {-expect:4d} had an illegal value" in out
    assert out.startswith("{    0,    0}:")


def test_pdgetrf_bad_context(sl, capfd):
    bad = sl.blacs_gridinit(2, 1)
    d = np.array([1, bad, 8, 8, 4, 4, 0, 0, 8], dtype=np.int32)
    assert _getrf_info(sl, 8, 8, 1, 1, d) == -602
    assert "{   -1,   -1}:  On entry to PDGETRF parameter number  602" in capfd.readouterr().out


def test_pdgetrs_argument_errors(sl, ctx):
    da = _desc(ctx)
    db = _desc(ctx, n=2)
    a = np.zeros((8, 8), order="F")
    b = np.zeros((8, 2), order="F")
    ip = np.ones(16, dtype=np.int32)
    assert sl.pdgetrs("X", 8, 2, a, 1, 1, da, ip, b, 1, 1, db) == -1
    assert sl.pdgetrs("N", -1, 2, a, 1, 1, da, ip, b, 1, 1, db) == -2
    assert sl.pdgetrs("N", 8, -1, a, 1, 1, da, ip, b, 1, 1, db) == -3
    assert sl.pdgetrs("N", 4, 2, a, 2, 1, da, ip, b, 1, 1, db) == -5
    assert sl.pdgetrs("N", 4, 2, a, 1, 2, da, ip, b, 1, 1, db) == -6
    assert sl.pdgetrs("N", 4, 2, a, 1, 1, da, ip, b, 2, 1, db) == -10
    assert sl.pdgetrs("N", 8, 2, a, 1, 1, _desc(ctx, mb=4, nb=2), ip, b, 1, 1, db) == -706
    assert sl.pdgetrs("N", 8, 2, a, 1, 1, da, ip, b, 1, 1, _desc(ctx, n=2, mb=2)) == -1206
    other = sl.blacs_gridinit(1, 1)
    assert sl.pdgetrs("N", 8, 2, a, 1, 1, da, ip, b, 1, 1, _desc(other, n=2)) == -1202
    assert sl.pdgetrs("N", 8, 2, a, 1, 1, da, ip, b, 1, 1, _desc(ctx, n=2, lld=4)) == -1209
    # quick return: nothing to do, no GPU needed
    assert sl.pdgetrs("N", 0, 2, a, 1, 1, da, ip, b, 1, 1, db) == 0


def test_pdgesv_argument_errors(sl, ctx):
    da = _desc(ctx)
    db = _desc(ctx, n=2)
    a = np.zeros((8, 8), order="F")
    b = np.zeros((8, 2), order="F")
    ip = np.zeros(16, dtype=np.int32)
    assert sl.pdgesv(-1, 2, a, 1, 1, da, ip, b, 1, 1, db) == -1
    assert sl.pdgesv(8, -1, a, 1, 1, da, ip, b, 1, 1, db) == -2
    assert sl.pdgesv(4, 2, a, 2, 1, da, ip, b, 1, 1, db) == -4
    assert sl.pdgesv(4, 2, a, 1, 2, da, ip, b, 1, 1, db) == -5
    assert sl.pdgesv(4, 2, a, 1, 1, da, ip, b, 2, 1, db) == -9
    assert sl.pdgesv(8, 2, a, 1, 1, da, ip, b, 1, 1, _desc(ctx, n=2, mb=2)) == -1106
    other = sl.blacs_gridinit(1, 1)
    assert sl.pdgesv(8, 2, a, 1, 1, da, ip, b, 1, 1, _desc(other, n=2)) == -1102
    assert sl.pdgesv(0, 2, a, 1, 1, da, ip, b, 1, 1, db) == 0


def test_quick_return_global_m_one(sl, ctx):
    # SRC/pdgetrf.f:201-203: DESCA(M_) == 1 sets IPIV(1) = 1 and returns.
    d = _desc(ctx, m=1, n=1, mb=1, nb=1, lld=1)
    a = np.array([[0.0]], order="F")
    ip = np.zeros(2, dtype=np.int32)
    assert sl.pdgetrf(1, 1, a, 1, 1, d, ip) == 0
    assert ip[0] == 1


def _no_gpu():
    try:
        import torch

        return not torch.cuda.is_available()
    except Exception:
        return True


@pytest.mark.skipif(not _no_gpu(), reason="checks the no-GPU error path")
def test_valid_call_without_gpu_fails_loudly(sl, ctx):
    d = _desc(ctx)
    info = _getrf_info(sl, 8, 8, 1, 1, d)
    assert info <= -10000  # never a silent CPU fallback


def test_pdgecon_validation_and_query(sl, ctx):
    # SRC/pdgecon.f:218-275: NORM -> -1, ANORM < 0 -> -7, LWORK -> -10, LIWORK -> -12
    n, nb = 8, 4
    d = _desc(ctx)
    a = np.zeros((8, 8), order="F")
    rc, info, w0, iw0 = sl.pdgecon("X", n, a, 1, 1, d, 1.0)
    assert info == -1
    rc, info, w0, iw0 = sl.pdgecon("1", n, a, 1, 1, d, -1.0)
    assert info == -7
    # workspace query: LWMIN = 2*NP + 2*NQ + max(2, NQ + NB), LIWMIN = max(1, NP)
    rc, info, w0, iw0 = sl.pdgecon("1", n, a, 1, 1, d, 1.0, lwork=-1)
    assert info == 0 and w0 == 2 * 8 + 2 * 8 + (8 + nb) and iw0 == 8
    rc, info, w0, iw0 = sl.pdgecon("I", n, a, 1, 1, d, 1.0, lwork=3)
    assert info == -10
    rc, info, w0, iw0 = sl.pdgecon("I", n, a, 1, 1, d, 1.0, liwork=1)
    assert info == -12
    # quick returns need no GPU: ANORM = 0 -> RCOND = 0
    rc, info, _, _ = sl.pdgecon("1", n, a, 1, 1, d, 0.0)
    assert info == 0 and rc == 0.0


def test_pdgetri_validation_and_query(sl, ctx):
    # SRC/pdgetri.f: IA/JA misaligned -> -4, MB != NB -> -506, LWORK -> -8, LIWORK -> -10
    d = _desc(ctx)
    a = np.zeros((8, 8), order="F")
    ip = np.arange(1, 17, dtype=np.int32)
    info, w0, iw0 = sl.pdgetri(4, a, 2, 1, d, ip)
    assert info == -4
    info, w0, iw0 = sl.pdgetri(8, a, 1, 1, _desc(ctx, mb=4, nb=2), ip)
    assert info == -506
    info, w0, iw0 = sl.pdgetri(8, a, 1, 1, d, ip, lwork=-1)
    assert info == 0 and w0 == 8 * 4 and iw0 == 8 + 4  # LWMIN = NP*NB, LIWMIN = NQ + NB
    info, w0, iw0 = sl.pdgetri(8, a, 1, 1, d, ip, lwork=1)
    assert info == -8
    info, w0, iw0 = sl.pdgetri(8, a, 1, 1, d, ip, liwork=1)
    assert info == -10
    assert sl.pdgetri(0, a, 1, 1, d, ip)[0] == 0


def test_alloc_failure_hook_state(sl):
    # the hook counts growths down to the one that fails, then disarms itself;
    # each call returns the previous state (-1: off or already fired)
    L = sl.lib()
    try:
        assert L.sl1x1_debug_fail_alloc(3) == -1
        assert L.sl1x1_debug_fail_alloc(0) == 3
        assert L.sl1x1_debug_fail_alloc(-5) == 0
        assert L.sl1x1_debug_fail_alloc(-1) == -1
    finally:
        L.sl1x1_debug_fail_alloc(-1)


def test_speed_settings_accept_any_value(sl):
    # speed-only settings clamp their argument and never fail
    L = sl.lib()
    for v in (-3, 0, 1, 8, 16, 99):
        L.sl1x1_set_copy_chunks(v)
    L.sl1x1_set_copy_chunks(8)
    L.sl1x1_set_lookahead(0)
    L.sl1x1_set_lookahead(1)
