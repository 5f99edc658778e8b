"""The oracle's PDGETRI restatement (oracle/sl_oracle.c, orc_pdgetri: PDTRTRI
and the blocked inv(A) L = inv(U) solve of SRC/pdgetri.f) against numpy's
inverse and LAPACK's DGETRI on the same factors, and its INFO on a singular
U. CPU only."""
import numpy as np
import pytest

scipy_lapack = pytest.importorskip("scipy.linalg.lapack")


@pytest.mark.parametrize("n,nb", [(1, 1), (5, 2), (64, 8), (200, 64), (333, 100), (130, 256)])
def test_getri_matches_inverse(orc, n, nb):
    rng = np.random.default_rng(n * 7 + nb)
    A = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    LU = np.asfortranarray(A.copy())
    ipiv, info = orc.pdgetrf(n, n, LU, nb=nb)
    assert info == 0
    rel = ipiv[:n] - 1
    info, X = orc.pdgetri(LU, rel, nb)
    assert info == 0
    eps = 2.0 ** -53
    R = A @ X - np.eye(n)
    assert np.abs(R).sum(1).max() / (np.abs(A).sum(1).max() * np.abs(X).sum(1).max() * n * eps) < 16
    # LAPACK's DGETRI on the same factors: the same matrix to rounding
    Xl, infol = scipy_lapack.dgetri(LU, rel)
    assert infol == 0
    assert np.abs(X - Xl).max() <= 1e-9 * np.abs(Xl).max()


def test_getri_singular_info(orc):
    n, nb = 50, 8
    rng = np.random.default_rng(5)
    A = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    A[:, 20] = 0.0
    LU = np.asfortranarray(A.copy())
    ipiv, k = orc.pdgetrf(n, n, LU, nb=nb)
    assert k == 21
    info, X = orc.pdgetri(LU, ipiv[:n] - 1, nb)
    assert info == 21
    np.testing.assert_array_equal(X, LU)
