"""CPU tests of the expert drivers' host logic: argument checks with the
reference's INFO codes and PXERBLA messages, workspace queries and the quick
returns that involve no GPU work (SRC/pdgerfs.f:334-461,
SRC/pdgesvx.f:455-665, SRC/pdgeequ.f:186-205, SRC/pdlaqge.f:160-215)."""
import numpy as np
import pytest


@pytest.fixture()
def ctx(sl):
    return sl.blacs_gridinit(1, 1)


def _desc(ctx, m=8, n=8, mb=4, nb=4, lld=8):
    return np.array([1, ctx, m, n, mb, nb, 0, 0, lld], dtype=np.int32)


def _gerfs(sl, ctx, trans="N", n=8, nrhs=2, ia=1, iaf=1, ib=1, ix=1, jb=1, jx=1, da=None,
           daf=None, db=None, dx=None, lwork=None, liwork=None):
    da = _desc(ctx) if da is None else da
    daf = _desc(ctx) if daf is None else daf
    db = _desc(ctx, n=4) if db is None else db
    dx = _desc(ctx, n=4) if dx is None else dx
    a = np.zeros((8, 8), order="F")
    af = np.zeros((8, 8), order="F")
    b = np.zeros((8, 4), order="F")
    x = np.zeros((8, 4), order="F")
    ipiv = np.arange(1, 17, dtype=np.int32)
    ferr = np.full(4, -7.0)
    berr = np.full(4, -7.0)
    info, w0, iw0 = sl.pdgerfs(trans, n, nrhs, a, ia, 1, da, af, iaf, 1, daf, ipiv, b, ib, jb, db, x,
                               ix, jx, dx, ferr, berr, lwork=lwork, liwork=liwork)
    return info, w0, iw0, ferr, berr


GERFS_CASES = [
    (dict(trans="X"), -1),
    (dict(n=-1), -2),
    (dict(nrhs=-1), -3),
    (dict(ia=2, n=4), -5),
    (dict(iaf=2, n=4), -9),
    (dict(ib=2, n=4), -14),
    (dict(ix=3, n=4), -18),
    (dict(jx=2, nrhs=1), -19),
    (dict(lwork=5), -24),
    (dict(liwork=1), -26),
]


@pytest.mark.parametrize("kw,expect", GERFS_CASES)
def test_pdgerfs_argument_errors(sl, ctx, capfd, kw, expect):
    info = _gerfs(sl, ctx, **kw)[0]
    assert info == expect
    assert f"On entry to PDGERFS parameter number {-expect:4d} had an illegal value" in \
        capfd.readouterr().out


def test_pdgerfs_descriptor_mismatch(sl, ctx):
    # MB_A != MB_AF -> -(1100+MB_); MB_A != NB_A -> -(700+NB_); MB_B != MB_X -> -(2000+MB_)
    assert _gerfs(sl, ctx, daf=_desc(ctx, mb=2, nb=4))[0] == -1105
    assert _gerfs(sl, ctx, da=_desc(ctx, mb=4, nb=2))[0] == -706
    assert _gerfs(sl, ctx, dx=_desc(ctx, n=4, mb=2))[0] == -2005


def test_pdgerfs_query_and_quick_return(sl, ctx):
    info, w0, iw0, _, _ = _gerfs(sl, ctx, lwork=-1)
    assert info == 0 and w0 == 3 * 8 and iw0 == 8  # LWMIN = 3 LOCr(N), LIWMIN = LOCr(N)
    # N <= 1: FERR = BERR = 0 from JB on, nothing else touched
    info, w0, iw0, ferr, berr = _gerfs(sl, ctx, n=1, nrhs=2, jb=2, jx=2)
    assert info == 0
    np.testing.assert_array_equal(ferr, [-7.0, 0.0, 0.0, -7.0])
    np.testing.assert_array_equal(berr, [-7.0, 0.0, 0.0, -7.0])


def _gesvx(sl, ctx, fact="N", trans="N", n=8, nrhs=2, ia=1, ja=1, iaf=1, equed="N", r=None, c=None,
           da=None, db=None, dx=None, lwork=None, liwork=None):
    da = _desc(ctx) if da is None else da
    db = _desc(ctx, n=4) if db is None else db
    dx = _desc(ctx, n=4) if dx is None else dx
    a = np.eye(8, order="F")
    af = np.zeros((8, 8), order="F")
    b = np.zeros((8, 4), order="F")
    x = np.zeros((8, 4), order="F")
    ipiv = np.zeros(16, dtype=np.int32)
    r = np.ones(8) if r is None else r
    c = np.ones(8) if c is None else c
    ferr = np.zeros(4)
    berr = np.zeros(4)
    return sl.pdgesvx(fact, trans, n, nrhs, a, ia, ja, da, af, iaf, 1, _desc(ctx), ipiv, equed, r, c,
                      b, 1, 1, db, x, 1, 1, dx, ferr, berr, lwork=lwork, liwork=liwork)


GESVX_CASES = [
    (dict(fact="X"), -1),
    (dict(trans="Q"), -2),
    (dict(ia=2, n=4), -6),
    (dict(ja=2, n=4), -7),
    (dict(iaf=2, n=4), -10),
    (dict(fact="F", equed="Z"), -13),
    (dict(fact="F", equed="R", r=np.array([1.0, 2, 3, 0, 1, 1, 1, 1])), -14),
    (dict(fact="F", equed="C", c=np.array([1.0, -2, 3, 1, 1, 1, 1, 1])), -15),
    (dict(lwork=10), -29),
    (dict(liwork=2), -31),
]


@pytest.mark.parametrize("kw,expect", GESVX_CASES)
def test_pdgesvx_argument_errors(sl, ctx, capfd, kw, expect):
    out = _gesvx(sl, ctx, **kw)
    assert out["info"] == expect
    assert f"On entry to PDGESVX parameter number {-expect:4d} had an illegal value" in \
        capfd.readouterr().out


def test_pdgesvx_descriptor_checks(sl, ctx):
    assert _gesvx(sl, ctx, da=_desc(ctx, mb=4, nb=2))["info"] == -806
    assert _gesvx(sl, ctx, db=_desc(ctx, n=4, mb=2))["info"] == -2006
    assert _gesvx(sl, ctx, dx=_desc(ctx, n=4, mb=2))["info"] == -2406


def test_pdgesvx_workspace_query(sl, ctx):
    # LWMIN = max(CONWRK, RFSWRK) on one process: CONWRK = 4N + max(2, NB, N+NB),
    # RFSWRK = 3N + 2N + ceil(N/NB)*NB (TRANS = 'N') or 5N (TRANS = 'T')
    n, nb = 8, 4
    out = _gesvx(sl, ctx, lwork=-1)
    assert out["info"] == 0 and out["work0"] == max(4 * n + n + nb, 5 * n + 2 * nb) and out["iwork0"] == n
    out = _gesvx(sl, ctx, trans="T", liwork=-1)
    assert out["info"] == 0 and out["work0"] == max(4 * n + n + nb, 5 * n)


def test_pdgesvx_n0_quick_return(sl, ctx):
    out = _gesvx(sl, ctx, n=0)
    assert out["info"] == 0 and out["rcond"] == 1.0 and out["equed"] == "N"


def test_pdgeequ_checks_and_quick_return(sl, ctx, capfd):
    d = _desc(ctx)
    a = np.zeros((8, 8), order="F")
    r, c = np.zeros(8), np.zeros(8)
    info, rc, cc, am = sl.pdgeequ(8, 8, a, 0, 1, d, r, c)
    assert info == -4  # IA < 1 (CHK1MAT position 4)
    assert "On entry to PDGEEQU parameter number    4" in capfd.readouterr().out
    info, rc, cc, am = sl.pdgeequ(0, 8, a, 1, 1, d, r, c)
    assert (info, rc, cc, am) == (0, 1.0, 1.0, 0.0)


def test_pdlaqge_decision_without_scaling(sl, ctx):
    d = _desc(ctx)
    a = np.full((8, 8), 3.0, order="F")
    r, c = np.ones(8), np.ones(8)
    assert sl.pdlaqge(8, 8, a, 1, 1, d, r, c, 1.0, 1.0, 1.0) == "N"
    assert sl.pdlaqge(0, 8, a, 1, 1, d, r, c, 1e-3, 1e-3, 1.0) == "N"
    np.testing.assert_array_equal(a, 3.0)
