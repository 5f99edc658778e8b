"""The ILP64 Fortran ABI (include/sl1x1_ilp64.h, libsl1x1gpu_ilp64.so): the
reference's entry points for callers built with 8-byte INTEGERs (its Int=long
build, README:145-154). CPU tests: the library exports every declared symbol,
NUMROC is exact beyond 2^31, the BLACS shim and DESCINIT agree with the 32-bit
library, argument errors give the 32-bit INFO codes (and an INTEGER outside the
32-bit range is an illegal argument), and IPIV is left alone on them. The GPU
test solves through both ABIs and compares the results bit for bit."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sl1x1_ilp64.h")
I64 = C.c_longlong


def declared():
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:void|double|sl_int64)\s+(\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def L64(sl):
    sl.lib()  # builds both libraries when needed
    return C.CDLL(sl._build.ilp64_path())


def ref(v):
    return C.byref(I64(v))


def desc64(ctx, m, n, mb, nb, lld):
    return np.array([1, ctx, m, n, mb, nb, 0, 0, lld], dtype=np.int64)


def p(a):
    return a.ctypes.data_as(C.c_void_p)


def test_exports_every_declared_symbol(L64, sl):
    names = declared()
    assert len(names) == 19 and "pdgesv_" in names and "numroc_" in names
    missing = [n for n in names if not hasattr(L64, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", sl._build.ilp64_path()], capture_output=True,
                         text=True).stdout
    assert set(names) <= {ln.split()[-1] for ln in out.splitlines() if ln.strip()}


def test_numroc_beyond_32_bits(L64):
    L64.numroc_.restype = I64
    assert L64.numroc_(ref(3_000_000_000), ref(64), ref(0), ref(0), ref(1)) == 3_000_000_000
    # TOOLS/numroc.f on 4 processes, N = 5e9 + 100, NB = 1000
    n, nb, P = 5_000_000_100, 1000, 4
    got = [L64.numroc_(ref(n), ref(nb), ref(q), ref(0), ref(P)) for q in range(P)]
    assert sum(got) == n
    nblocks = n // nb
    for q in range(P):
        r = (nblocks // P) * nb
        extra = nblocks % P
        r += nb if q < extra else (n % nb if q == extra else 0)
        assert got[q] == r


def test_blacs_and_descinit(L64, sl):
    ctxt = I64(0)
    L64.blacs_gridinit_(C.byref(ctxt), b"R", ref(1), ref(1), C.c_size_t(1))
    pr, pc, r, c = I64(), I64(), I64(), I64()
    L64.blacs_gridinfo_(C.byref(ctxt), C.byref(pr), C.byref(pc), C.byref(r), C.byref(c))
    assert (pr.value, pc.value, r.value, c.value) == (1, 1, 0, 0)
    # the contexts are the 32-bit library's own
    assert sl.blacs_gridinfo(int(ctxt.value)) == (1, 1, 0, 0)
    d = np.zeros(9, np.int64)
    info = I64(7)
    L64.descinit_(p(d), ref(300), ref(200), ref(32), ref(32), ref(0), ref(0), C.byref(ctxt), ref(300),
                  C.byref(info))
    assert info.value == 0
    np.testing.assert_array_equal(d, [1, ctxt.value, 300, 200, 32, 32, 0, 0, 300])
    L64.descinit_(p(d), ref(300), ref(200), ref(0), ref(32), ref(0), ref(0), C.byref(ctxt), ref(300),
                  C.byref(info))
    assert info.value == -4
    L64.descinit_(p(d), ref(300), ref(200), ref(32), ref(32), ref(0), ref(0), C.byref(ctxt),
                  ref(1 << 40), C.byref(info))
    assert info.value == -9  # LLD outside the 32-bit range
    me, np_ = I64(), I64()
    L64.blacs_pinfo_(C.byref(me), C.byref(np_))
    assert (me.value, np_.value) == (0, 1)
    L64.blacs_gridexit_(C.byref(ctxt))
    assert sl.blacs_gridinfo(int(ctxt.value)) == (-1, -1, -1, -1)


def _pdgesv64(L64, n, nrhs, A, da, ipiv, B, db, ia=1, ja=1):
    info = I64(99)
    L64.pdgesv_(ref(n), ref(nrhs), p(A), ref(ia), ref(ja), p(da), p(ipiv), p(B), ref(ia), ref(1),
                p(db), C.byref(info))
    return info.value


def test_argument_errors_match_the_32_bit_codes(L64, sl):
    ctx = sl.blacs_gridinit(1, 1)
    n, nb = 40, 8
    A = np.asfortranarray(np.eye(n))
    B = np.asfortranarray(np.ones((n, 1)))
    ipiv = np.full(n + nb, -5, np.int64)
    da, db = desc64(ctx, n, n, nb, nb, n), desc64(ctx, n, 1, nb, nb, n)
    d32a = np.array(da, np.int32)
    d32b = np.array(db, np.int32)
    ip32 = np.zeros(n + nb, np.int32)
    for bad_n in (-1,):
        got = _pdgesv64(L64, bad_n, 1, A, da, ipiv, B, db)
        want = sl.pdgesv(bad_n, 1, A, 1, 1, d32a, ip32, B, 1, 1, d32b)
        assert got == want == -1
    # an IA the 32-bit routines reject, and a context that is not a grid
    assert _pdgesv64(L64, n, 1, A, da, ipiv, B, db, ia=3) == sl.pdgesv(n, 1, A, 3, 1, d32a, ip32, B, 3, 1, d32b)
    bad = da.copy()
    bad[1] = 12345
    assert _pdgesv64(L64, n, 1, A, bad, ipiv, B, db) == sl.pdgesv(
        n, 1, A, 1, 1, np.array(bad, np.int32), ip32, B, 1, 1, d32b)
    # INTEGERs outside the 32-bit range: the argument's position (descriptor: 100 * pos + entry)
    assert _pdgesv64(L64, 1 << 33, 1, A, da, ipiv, B, db) == -1
    big = da.copy()
    big[2] = 1 << 35
    assert _pdgesv64(L64, n, 1, A, big, ipiv, B, db) == -603
    info = I64(0)
    L64.pdgetrf_(ref(n), ref(n), p(A), ref(1), ref(1 << 32), p(da), p(ipiv), C.byref(info))
    assert info.value == -5
    np.testing.assert_array_equal(ipiv, -5)  # no IPIV entry written on argument errors
    np.testing.assert_array_equal(A, np.eye(n))


@pytest.mark.gpu
def test_pdgesv_through_both_abis_bitwise(L64, sl, orc, gpu_required):
    ctx = sl.blacs_gridinit(1, 1)
    n, nrhs, nb = 300, 3, 32
    rng = np.random.default_rng(64)
    A0 = np.asfortranarray(rng.uniform(-0.5, 0.5, (n, n)))
    B0 = np.asfortranarray(rng.uniform(-0.5, 0.5, (n, nrhs)))
    A32, B32 = A0.copy(order="F"), B0.copy(order="F")
    ip32 = np.zeros(n + nb, np.int32)
    d32a = np.array([1, ctx, n, n, nb, nb, 0, 0, n], np.int32)
    d32b = np.array([1, ctx, n, nrhs, nb, nb, 0, 0, n], np.int32)
    assert sl.pdgesv(n, nrhs, A32, 1, 1, d32a, ip32, B32, 1, 1, d32b) == 0
    A64, B64 = A0.copy(order="F"), B0.copy(order="F")
    ip64 = np.full(n + nb, -7, np.int64)
    assert _pdgesv64(L64, n, nrhs, A64, np.array(d32a, np.int64), ip64, B64,
                     np.array(d32b, np.int64)) == 0
    np.testing.assert_array_equal(ip64[:n], ip32[:n])
    np.testing.assert_array_equal(ip64[n:], -7)
    np.testing.assert_array_equal(A64, A32)
    np.testing.assert_array_equal(B64, B32)
    assert orc.sresid(A0, B0, B64) < 16.0


def test_workspace_queries_match_the_32_bit_library(L64, sl):
    # LWORK = LIWORK = -1: WORK(1) and IWORK(1) report the minimal sizes, no device work
    ctx = sl.blacs_gridinit(1, 1)
    n, nb = 500, 64
    A = np.asfortranarray(np.eye(n))
    d32 = np.array([1, ctx, n, n, nb, nb, 0, 0, n], np.int32)
    d64 = np.array(d32, np.int64)
    rc32, info32, w32, iw32 = sl.pdgecon("1", n, A, 1, 1, d32, 1.0, lwork=-1, liwork=-1)
    work = np.zeros(4)
    iwork = np.zeros(4, np.int64)
    rc, info = C.c_double(), I64(5)
    L64.pdgecon_(b"1", ref(n), p(A), ref(1), ref(1), p(d64), C.byref(C.c_double(1.0)), C.byref(rc),
                 p(work), ref(-1), p(iwork), ref(-1), C.byref(info), C.c_size_t(1))
    assert info.value == info32 == 0
    assert work[0] == w32 and iwork[0] == iw32 > 0
    ipiv32 = np.arange(1, n + nb + 1, dtype=np.int32)
    info32, w32, iw32 = sl.pdgetri(n, A, 1, 1, d32, ipiv32, lwork=-1, liwork=-1)
    ipiv64 = np.arange(1, n + nb + 1, dtype=np.int64)
    work[:] = 0
    iwork[:] = 0
    L64.pdgetri_(ref(n), p(A), ref(1), ref(1), p(d64), p(ipiv64), p(work), ref(-1), p(iwork), ref(-1),
                 C.byref(info))
    assert info.value == info32 == 0
    assert work[0] == w32 and iwork[0] == iw32 > 0
    # argument errors: the 32-bit codes
    L64.pdgetri_(ref(-3), p(A), ref(1), ref(1), p(d64), p(ipiv64), p(work), ref(10), p(iwork), ref(10),
                 C.byref(info))
    assert info.value == sl.pdgetri(-3, A, 1, 1, d32, ipiv32, lwork=10, liwork=10)[0] == -1
