"""CPU tests of the oracle's expert-driver restatement (PDGEEQU, PDLAQGE,
PDGECON, PDGERFS, PDGESVX on one process).

Pins: LAPACK DGEEQU / DGESVX from scipy (same equilibration arithmetic, so
R, C, ROWCND, COLCND, AMAX and EQUED must agree bit for bit; the solution,
RCOND, FERR and BERR agree to rounding / estimator noise), plus the defining
properties of PDGERFS: BERR is the componentwise backward error of the
returned X, and FERR bounds the true forward error.
"""
import numpy as np
import pytest
import scipy.linalg.lapack as lapack


def badly_scaled(rng, n, rows=1e-6, cols=1e5):
    A = rng.uniform(-1.0, 1.0, (n, n))
    A *= np.exp(rng.uniform(np.log(rows), 0.0, n))[:, None]
    A *= np.exp(rng.uniform(0.0, np.log(cols), n))[None, :]
    return np.asfortranarray(A)


@pytest.mark.parametrize("n,seed", [(1, 0), (7, 1), (40, 2), (128, 3)])
def test_pdgeequ_matches_lapack_bitwise(orc, n, seed):
    rng = np.random.default_rng(seed)
    A = badly_scaled(rng, n)
    R, C, rc, cc, am, info = orc.pdgeequ(A)
    r2, c2, rc2, cc2, am2, info2 = lapack.dgeequ(A)
    assert info == info2 == 0
    np.testing.assert_array_equal(R, r2)
    np.testing.assert_array_equal(C, c2)
    assert (rc, cc, am) == (rc2, cc2, am2)


def test_pdgeequ_zero_row_and_column(orc):
    rng = np.random.default_rng(5)
    A = np.asfortranarray(rng.uniform(-1, 1, (6, 5)))
    A[3, :] = 0.0
    assert orc.pdgeequ(A)[5] == 4  # first zero row
    A = np.asfortranarray(rng.uniform(-1, 1, (6, 5)))
    A[:, 2] = 0.0
    assert orc.pdgeequ(A)[5] == 6 + 3  # M + first zero column
    assert lapack.dgeequ(A)[5] == 9


@pytest.mark.parametrize("rows,cols,expect", [(1.0, 1.0, "N"), (1.0, 1e4, "C"), (1e-4, 1.0, "R"),
                                              (1e-4, 1e4, "B")])
def test_pdlaqge_decision_and_scaling(orc, rows, cols, expect):
    rng = np.random.default_rng(11)
    n = 20
    A = np.asfortranarray(rng.uniform(0.5, 1.0, (n, n)))
    A[: n // 2, :] *= rows
    A[:, : n // 2] *= cols
    R, C, rc, cc, am, info = orc.pdgeequ(A)
    As, eq = orc.pdlaqge(A, R, C, rc, cc, am)
    assert eq == expect
    ref = A.copy()
    if eq in "RB":
        ref = ref * (R[:, None] if eq == "R" else 1.0)
    if eq == "C":
        ref = C[None, :] * A
    if eq == "B":
        ref = (C[None, :] * R[:, None]) * A
    np.testing.assert_array_equal(As, ref)


@pytest.mark.parametrize("trans", ["N", "T"])
@pytest.mark.parametrize("fact", ["N", "E"])
def test_pdgesvx_matches_lapack_dgesvx(orc, fact, trans):
    rng = np.random.default_rng(21)
    n, nrhs = 60, 3
    A = badly_scaled(rng, n)
    B = np.asfortranarray(rng.uniform(-1, 1, (n, nrhs)))
    r = orc.pdgesvx(fact, trans, A, B, nb=16)
    out = lapack.dgesvx(A, B, fact=fact, trans=trans)
    as_, lu, ipiv, equed, rs, cs, bs, x, rcond, ferr, berr, info = out
    assert r["info"] == info == 0
    assert r["equed"] == equed.decode()
    if fact == "E":
        np.testing.assert_array_equal(r["R"], rs)
        np.testing.assert_array_equal(r["C"], cs)
        np.testing.assert_array_equal(r["A"], as_)
        np.testing.assert_array_equal(r["B"], bs)
    np.testing.assert_array_equal(r["ipiv"], ipiv + 1)  # same partial pivoting
    # the condition estimate and error bounds come from the same estimator
    assert 0.5 < r["rcond"] / rcond < 2.0
    np.testing.assert_allclose(r["ferr"], ferr, rtol=0.5)
    assert np.all(r["berr"] <= 4 * np.finfo(float).eps)
    scale = np.abs(x).max(axis=0)
    assert np.all(np.abs(r["X"] - x).max(axis=0) <= 10 * np.maximum(ferr, r["ferr"]) * scale)


def _true_solution(A, B):
    """X refined in extended precision (long double residuals)."""
    X = np.linalg.solve(A, B)
    Al, Bl = A.astype(np.longdouble), B.astype(np.longdouble)
    for _ in range(3):
        Rl = Bl - Al @ X.astype(np.longdouble)
        X = X + np.linalg.solve(A, Rl.astype(np.float64))
    return X


@pytest.mark.parametrize("trans", ["N", "T"])
def test_pdgerfs_backward_and_forward_error(orc, trans):
    rng = np.random.default_rng(31)
    n, nrhs = 50, 2
    A = np.asfortranarray(orc.gen_conditioned(n, 1e6, nrefl=8, seed=4))
    B = np.asfortranarray(rng.uniform(-1, 1, (n, nrhs)))
    AF = np.asfortranarray(A.copy())
    ipiv, info = orc.pdgetrf(n, n, AF, nb=16)
    assert info == 0
    # a deliberately rough starting solution: one FP32-accurate solve
    X0 = np.asfortranarray(np.linalg.solve(A.astype(np.float32), B.astype(np.float32)).astype(np.float64))
    X, ferr, berr = orc.pdgerfs(trans, A, AF, ipiv, B, X0)
    op = A if trans == "N" else A.T
    # BERR is the componentwise backward error of the returned X (up to the
    # rounding of the last residual)
    for k in range(nrhs):
        r = B[:, k] - op @ X[:, k]
        w = np.abs(B[:, k]) + np.abs(op) @ np.abs(X[:, k])
        assert np.max(np.abs(r) / w) <= 2 * berr[k] + 4 * np.finfo(float).eps
    assert np.all(berr < 1e-15)
    Xt = _true_solution(op, B)
    fwd = np.abs(X - Xt).max(axis=0) / np.abs(X).max(axis=0)
    assert np.all(fwd <= ferr), (fwd, ferr)
    assert np.all(ferr < 1e-6)


def test_pdgesvx_singular_and_rcond(orc):
    n = 12
    rng = np.random.default_rng(41)
    A = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    A[:, 5] = 0.0
    B = np.asfortranarray(rng.uniform(-1, 1, (n, 1)))
    r = orc.pdgesvx("N", "N", A, B, nb=4)
    assert r["info"] == 6 and r["rcond"] == 0.0
    # numerically singular (two equal columns): RCOND < eps gives INFO = IA + N,
    # unless elimination hits an exact zero pivot first (INFO = that column)
    A = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    A[:, 7] = A[:, 2]
    r = orc.pdgesvx("N", "N", A, B, nb=4)
    assert r["info"] in (n + 1, 8)
    if r["info"] == n + 1:
        assert r["rcond"] < np.finfo(float).eps / 2
