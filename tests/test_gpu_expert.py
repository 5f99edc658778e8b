"""GPU parity tests of the expert drivers through the C ABI against the CPU
oracle (C restatement of SRC/pdgeequ.f, pdlaqge.f, pdgecon.f, pdgerfs.f,
pdgesvx.f on one process).

Bit-exact where the arithmetic is exact in any order (scale factors, EQUED,
the equilibrated A and B); IPIV compared with near-tie replay as for PDGETRF;
X within 10 x FERR of the oracle's X; RCOND and FERR within a factor 2 and
1.5 (same estimator, different rounding of the solves); BERR at the
unit-roundoff level like the oracle's.
"""
import numpy as np
import pytest

from lu_helpers import compare_ipiv

pytestmark = pytest.mark.gpu
EPS = np.finfo(float).eps / 2


@pytest.fixture()
def ctx(sl):
    return sl.blacs_gridinit(1, 1)


def desc(ctx, m, n, nb, lld=None):
    return np.array([1, ctx, m, n, nb, nb, 0, 0, max(1, lld if lld is not None else m)], np.int32)


def badly_scaled(rng, n, rows=1e-6, cols=1e5):
    A = rng.uniform(-1.0, 1.0, (n, n))
    A *= np.exp(rng.uniform(np.log(rows), 0.0, n))[:, None]
    A *= np.exp(rng.uniform(0.0, np.log(cols), n))[None, :]
    return np.asfortranarray(A)


@pytest.mark.parametrize("m,n", [(1, 1), (17, 9), (300, 300), (1000, 700)])
def test_pdgeequ_bitwise(sl, orc, ctx, gpu_required, m, n):
    rng = np.random.default_rng(m + n)
    A = np.asfortranarray(rng.uniform(-1, 1, (m, n)) * np.exp(rng.uniform(-12, 12, (m, 1))))
    R, C, rc, cc, am, info = orc.pdgeequ(A)
    r = np.zeros(m)
    c = np.zeros(n)
    info2, rc2, cc2, am2 = sl.pdgeequ(m, n, A, 1, 1, desc(ctx, m, n, 16), r, c)
    assert info2 == info == 0
    np.testing.assert_array_equal(r, R)
    np.testing.assert_array_equal(c, C)
    assert (rc2, cc2, am2) == (rc, cc, am)


def test_pdgeequ_zero_row_column_and_offsets(sl, orc, ctx, gpu_required):
    rng = np.random.default_rng(3)
    A = np.asfortranarray(rng.uniform(-1, 1, (40, 30)))
    A[17, :] = 0.0
    r, c = np.zeros(40), np.zeros(30)
    assert sl.pdgeequ(40, 30, A, 1, 1, desc(ctx, 40, 30, 8), r, c)[0] == 18
    A = np.asfortranarray(rng.uniform(-1, 1, (40, 30)))
    A[:, 11] = 0.0
    assert sl.pdgeequ(40, 30, A, 1, 1, desc(ctx, 40, 30, 8), r, c)[0] == 40 + 12
    # sub(A) at (IA, JA) = (9, 5): R(9..), C(5..) written, the rest untouched
    A = np.asfortranarray(rng.uniform(-1, 1, (40, 30)))
    r, c = np.full(40, -1.0), np.full(30, -1.0)
    info, rc, cc, am = sl.pdgeequ(20, 10, A, 9, 5, desc(ctx, 40, 30, 4), r, c)
    R, C, rc0, cc0, am0, info0 = orc.pdgeequ(np.asfortranarray(A[8:28, 4:14]))
    assert info == info0 == 0
    np.testing.assert_array_equal(r[8:28], R)
    np.testing.assert_array_equal(c[4:14], C)
    assert np.all(r[:8] == -1.0) and np.all(r[28:] == -1.0) and np.all(c[14:] == -1.0)


@pytest.mark.parametrize("rows,cols,expect", [(1.0, 1e4, "C"), (1e-4, 1.0, "R"), (1e-4, 1e4, "B")])
def test_pdlaqge_bitwise(sl, orc, ctx, gpu_required, rows, cols, expect):
    rng = np.random.default_rng(9)
    n = 64
    A = np.asfortranarray(rng.uniform(0.5, 1.0, (n, n)))
    A[: n // 2, :] *= rows
    A[:, : n // 2] *= cols
    R, C, rc, cc, am, info = orc.pdgeequ(A)
    ref, eq = orc.pdlaqge(A, R, C, rc, cc, am)
    a = np.array(A, order="F")
    eq2 = sl.pdlaqge(n, n, a, 1, 1, desc(ctx, n, n, 16), np.ascontiguousarray(R),
                     np.ascontiguousarray(C), rc, cc, am)
    assert eq2 == eq == expect
    np.testing.assert_array_equal(a, ref)


def _factor(sl, ctx, A, nb):
    n = A.shape[0]
    AF = np.array(A, order="F")
    ipiv = np.zeros(n + nb, np.int32)
    assert sl.pdgetrf(n, n, AF, 1, 1, desc(ctx, n, n, nb), ipiv) == 0
    return AF, ipiv


@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("n,nrhs,nb", [(2, 1, 2), (65, 3, 16), (500, 2, 64), (1200, 1, 128)])
def test_pdgerfs_matches_oracle(sl, orc, ctx, gpu_required, trans, n, nrhs, nb):
    rng = np.random.default_rng(n + nrhs)
    A = np.asfortranarray(orc.gen_conditioned(n, 1e5, nrefl=8, seed=n)) if n <= 500 else \
        np.asfortranarray(rng.uniform(-0.5, 0.5, (n, n)))
    B = np.asfortranarray(rng.uniform(-1, 1, (n, nrhs)))
    AF, ipiv = _factor(sl, ctx, A, nb)
    # a rough starting solution (FP32 solve) so that refinement has work to do
    X0 = np.asfortranarray(np.linalg.solve(A.astype(np.float32), B.astype(np.float32)).astype(np.float64))
    Xo, ferr_o, berr_o = orc.pdgerfs(trans, A, AF, ipiv, B, X0)
    X = np.array(X0, order="F")
    ferr, berr = np.zeros(nrhs), np.zeros(nrhs)
    d = desc(ctx, n, n, nb)
    db = desc(ctx, n, nrhs, nb)
    info, w0, iw0 = sl.pdgerfs(trans, n, nrhs, A, 1, 1, d, AF, 1, 1, d, ipiv, B, 1, 1, db, X, 1, 1,
                               db, ferr, berr)
    assert info == 0 and w0 == 3 * n and iw0 == n
    # the oracle refines with the GPU factors too; its stopping point can sit a
    # hair above 4 eps on these kappa = 1e5 inputs
    assert np.all(berr <= 4 * EPS) and np.all(berr_o <= 8 * EPS)
    assert np.all(ferr > 0)
    np.testing.assert_allclose(ferr, ferr_o, rtol=0.5)
    scale = np.abs(Xo).max(axis=0)
    assert np.all(np.abs(X - Xo).max(axis=0) <= 10 * np.maximum(ferr, ferr_o) * scale)


def test_pdgerfs_offsets_and_ferr_index(sl, orc, ctx, gpu_required):
    # sub-matrices at (IA, JA) = (5, 5) of a 40 x 40 array (NB 4), B/X at column 3;
    # FERR/BERR are indexed from JB as the reference does
    rng = np.random.default_rng(77)
    n, nrhs, nb = 32, 2, 4
    Abig = np.asfortranarray(rng.uniform(-1, 1, (40, 40)))
    A = np.asfortranarray(Abig[4:36, 4:36])
    AF, ipiv_rel = _factor(sl, ctx, A, nb)
    AFbig = np.asfortranarray(np.zeros((40, 40)))
    AFbig[4:36, 4:36] = AF
    ipiv = np.zeros(48, np.int32)
    ipiv[4:36] = ipiv_rel[:n] + 4
    Bbig = np.asfortranarray(rng.uniform(-1, 1, (40, 6)))
    Xbig = np.asfortranarray(np.zeros((40, 6)))
    Xbig[4:36, 2:4] = np.linalg.solve(A, Bbig[4:36, 2:4]) * (1 + 1e-9)
    ferr, berr = np.full(6, -1.0), np.full(6, -1.0)
    d = desc(ctx, 40, 40, nb)
    db = desc(ctx, 40, 6, nb)
    info, _, _ = sl.pdgerfs("N", n, nrhs, Abig, 5, 5, d, AFbig, 5, 5, d, ipiv, Bbig, 5, 3, db, Xbig, 5,
                            3, db, ferr, berr)
    assert info == 0
    assert np.all(ferr[[0, 1, 4, 5]] == -1.0) and np.all(berr[[0, 1, 4, 5]] == -1.0)
    assert np.all(berr[2:4] <= 4 * EPS) and np.all(ferr[2:4] > 0)
    np.testing.assert_allclose(Xbig[4:36, 2:4], np.linalg.solve(A, Bbig[4:36, 2:4]), rtol=0,
                               atol=1e-10)


def _gesvx_gpu(sl, ctx, fact, trans, A, B, nb, AF=None, ipiv=None, equed="N", R=None, C=None):
    n, nrhs = B.shape
    a = np.array(A, order="F")
    b = np.array(B, order="F")
    af = np.zeros((n, n), order="F") if AF is None else np.array(AF, order="F")
    ip = np.zeros(n + nb, np.int32) if ipiv is None else np.array(ipiv, np.int32)
    r = np.zeros(n) if R is None else np.array(R)
    c = np.zeros(n) if C is None else np.array(C)
    x = np.zeros((n, nrhs), order="F")
    ferr, berr = np.zeros(nrhs), np.zeros(nrhs)
    d = desc(ctx, n, n, nb)
    db = desc(ctx, n, nrhs, nb)
    out = sl.pdgesvx(fact, trans, n, nrhs, a, 1, 1, d, af, 1, 1, d, ip, equed, r, c, b, 1, 1, db, x, 1,
                     1, db, ferr, berr)
    out.update(A=a, B=b, AF=af, ipiv=ip, R=r, C=c, X=x, ferr=ferr, berr=berr)
    return out


@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("fact", ["N", "E"])
@pytest.mark.parametrize("n,nrhs,nb", [(60, 3, 16), (513, 2, 64)])
def test_pdgesvx_matches_oracle(sl, orc, ctx, gpu_required, fact, trans, n, nrhs, nb):
    rng = np.random.default_rng(1000 + n)
    A = badly_scaled(rng, n)
    B = np.asfortranarray(rng.uniform(-1, 1, (n, nrhs)))
    o = orc.pdgesvx(fact, trans, A, B, nb=nb)
    g = _gesvx_gpu(sl, ctx, fact, trans, A, B, nb)
    assert g["info"] == o["info"] == 0
    assert g["equed"] == o["equed"]
    if fact == "E":
        assert o["equed"] == "B"
        np.testing.assert_array_equal(g["R"], o["R"])
        np.testing.assert_array_equal(g["C"], o["C"])
        np.testing.assert_array_equal(g["A"], o["A"])
        np.testing.assert_array_equal(g["B"], o["B"])
    bad, ties = compare_ipiv(orc, o["A"] if fact == "E" else A, g["ipiv"][:n], nb)
    assert bad == 0, ties
    assert 0.5 < g["rcond"] / o["rcond"] < 2.0
    np.testing.assert_allclose(g["ferr"], o["ferr"], rtol=0.5)
    assert np.all(g["berr"] <= 4 * EPS)
    scale = np.abs(o["X"]).max(axis=0)
    assert np.all(np.abs(g["X"] - o["X"]).max(axis=0) <= 10 * np.maximum(g["ferr"], o["ferr"]) * scale)


@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("equed", ["N", "R", "C", "B"])
def test_pdgesvx_factored_and_equilibrated_input(sl, orc, ctx, gpu_required, trans, equed):
    # FACT = 'F': caller supplies AF, IPIV and (for EQUED != 'N') the scale
    # factors with A already equilibrated
    rng = np.random.default_rng(5)
    n, nrhs, nb = 90, 2, 16
    A0 = badly_scaled(rng, n)
    R, C, rc, cc, am, _ = orc.pdgeequ(A0)
    A = np.array(A0, order="F")
    if equed in "RB":
        A = R[:, None] * A
    if equed in "CB":
        A = A * C[None, :]
    A = np.asfortranarray(A)
    AF, ipiv = _factor(sl, ctx, A, nb)
    B = np.asfortranarray(rng.uniform(-1, 1, (n, nrhs)))
    o = orc.pdgesvx("F", trans, A, B, AF=AF, ipiv=ipiv[:n], equed=equed, R=R, Cv=C, nb=nb)
    g = _gesvx_gpu(sl, ctx, "F", trans, A, B, nb, AF=AF, ipiv=ipiv, equed=equed, R=R, C=C)
    assert g["info"] == o["info"] == 0 and g["equed"] == equed
    np.testing.assert_array_equal(g["B"], o["B"])
    np.testing.assert_array_equal(g["AF"], AF)
    assert 0.5 < g["rcond"] / o["rcond"] < 2.0
    np.testing.assert_allclose(g["ferr"], o["ferr"], rtol=0.5)
    scale = np.abs(o["X"]).max(axis=0)
    assert np.all(np.abs(g["X"] - o["X"]).max(axis=0) <= 10 * np.maximum(g["ferr"], o["ferr"]) * scale)
    # X solves the original (unequilibrated) system op(A0) X = B0 when the
    # caller undoes its own scaling of B -- here: residual of the equilibrated system
    op = A if trans == "N" else A.T
    bs = g["B"]
    xs = g["X"] / (C[:, None] if (trans == "N" and equed in "CB") else 1.0)
    xs = xs / (R[:, None] if (trans == "T" and equed in "RB") else 1.0)
    resid = np.abs(op @ xs - bs) / (np.abs(op) @ np.abs(xs) + np.abs(bs))
    assert resid.max() <= 1e-13


def test_pdgesvx_singular(sl, orc, ctx, gpu_required):
    rng = np.random.default_rng(8)
    n, nb = 40, 8
    A = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    A[:, 13] = 0.0
    B = np.asfortranarray(rng.uniform(-1, 1, (n, 1)))
    g = _gesvx_gpu(sl, ctx, "N", "N", A, B, nb)
    o = orc.pdgesvx("N", "N", A, B, nb=nb)
    assert g["info"] == o["info"] == 14 and g["rcond"] == 0.0
    # numerically singular: two equal columns
    A = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    A[:, 20] = A[:, 3]
    g = _gesvx_gpu(sl, ctx, "N", "N", A, B, nb)
    assert g["info"] in (n + 1, 21)
    if g["info"] == n + 1:
        assert g["rcond"] < EPS


def test_device_forms(sl, orc, gpu_required):
    import torch

    rng = np.random.default_rng(12)
    n, nrhs = 300, 2
    A = badly_scaled(rng, n)
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dR = torch.zeros(n, dtype=torch.float64, device="cuda")
    dC = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    info, rc, cc, am = sl.dgeequ_dev(n, n, dA.data_ptr(), n, dR.data_ptr(), dC.data_ptr())
    R, C, rc0, cc0, am0, info0 = orc.pdgeequ(A)
    assert info == info0 == 0 and (rc, cc, am) == (rc0, cc0, am0)
    np.testing.assert_array_equal(dR.cpu().numpy(), R)
    np.testing.assert_array_equal(dC.cpu().numpy(), C)
    # refinement on device data (LAPACK 1-based pivots)
    A = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    B = np.asfortranarray(rng.uniform(-1, 1, (n, nrhs)))
    dA = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    dAF = dA.clone()
    dpiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    assert sl.dgetrf_dev(n, n, dAF.data_ptr(), n, dpiv.data_ptr()) == 0
    dB = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    dX = (dB.clone() * 0.0)
    X0 = np.linalg.solve(A.astype(np.float32), B.astype(np.float32)).astype(np.float64)
    dX.copy_(torch.from_numpy(np.ascontiguousarray(X0.T)))
    torch.cuda.synchronize()
    info, ferr, berr = sl.dgerfs_dev("N", n, nrhs, dA.data_ptr(), n, dAF.data_ptr(), n, dpiv.data_ptr(),
                                     dB.data_ptr(), n, dX.data_ptr(), n)
    assert info == 0 and np.all(berr <= 4 * EPS) and np.all(ferr > 0)
    X = dX.cpu().numpy().T
    np.testing.assert_allclose(X, np.linalg.solve(A, B), rtol=0, atol=1e-11)
