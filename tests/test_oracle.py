"""Pin the CPU oracle (C restatement of the reference's 1x1 LU path).

The reference itself cannot be compiled here (Fortran 77 + MPI, no compiler),
so the oracle is checked against: the EXAMPLE known-answer system, the
tester generator's own integer arithmetic, LAPACK DGETRF/DGETRS from the host
BLAS (same partial-pivoting rule), and the tester's residual thresholds on the
LU.dat sizes.
"""
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_generator_matches_fortran_integer_halves(orc):
    g = json.load(open(os.path.join(GOLD, "pdmatgen.json")))
    for seed, vals in g["values"].items():
        seed = int(seed)
        # a 64 x 1 matrix walks the stream in order; kind 0 is 1 - 2*PDRAND
        col = orc.matgen(64, 1, seed, kind=0)[:, 0]
        np.testing.assert_array_equal(col, 1.0 - 2.0 * np.array(vals))
        col1 = orc.matgen(64, 1, seed, kind=1)[:, 0]
        np.testing.assert_array_equal(col1, 0.5 - np.array(vals))


def test_generator_column_major_and_blocks(orc):
    M, N = 37, 11
    full = orc.matgen(M, N, 100)
    g = json.load(open(os.path.join(GOLD, "pdmatgen.json")))
    # entry (i, j) is draw number j*M + i of the stream
    flat = full.flatten(order="F")
    np.testing.assert_array_equal(flat[:64], 1.0 - 2.0 * np.array(g["values"]["100"]))
    blk = orc.matgen(M, N, 100, i0=5, j0=3, nrows=20, ncols=6)
    np.testing.assert_array_equal(blk, full[5:25, 3:9])
    d = orc.matgen(M, N, 100, diag=True)
    for i in range(min(M, N)):
        assert d[i, i] == abs(full[i, i]) + max(M, N)
    assert np.all(full > -1.0) and np.all(full <= 1.0)


def test_example_known_answer(orc):
    d = json.load(open(os.path.join(GOLD, "dscaex.json")))
    n = d["n"]
    A = np.array(d["a_colmajor"], dtype=np.float64).reshape((n, n), order="F")
    B = np.array(d["b"], dtype=np.float64).reshape((n, 1), order="F")
    LU, ipiv, X, info = orc.solve_reference(A, B, nb=d["nb"])
    assert info == 0
    np.testing.assert_allclose(X[:, 0], d["x_exact"], rtol=1e-13)
    # EXAMPLE/pdscaex.f:181-191: residual / (||A|| ||x|| eps N) < 10
    assert orc.sresid(A, B, X) < d["threshold"]


LU_DAT_MN = [(4, 4), (10, 12), (17, 13), (13, 13)]
LU_DAT_NB = [2, 3, 4]


@pytest.mark.parametrize("m,n", LU_DAT_MN)
@pytest.mark.parametrize("nb", LU_DAT_NB)
def test_oracle_pivots_equal_lapack_lu_dat(orc, m, n, nb):
    A0 = orc.matgen(m, n, 100)
    A = np.asfortranarray(A0.copy())
    ipiv, info = orc.pdgetrf(m, n, A, nb=nb)
    LUl, ipl, infol = orc.lapack_dgetrf(A0)
    assert info == infol == 0
    mn = min(m, n)
    np.testing.assert_array_equal(ipiv[:mn], ipl)
    np.testing.assert_allclose(A, LUl, rtol=0, atol=1e-13)
    assert orc.fresid(A, ipiv[:mn], A0) < 1.0  # LU.dat THRESH


@pytest.mark.parametrize("n,nb", [(300, 32), (257, 64), (129, 1), (200, 256)])
def test_oracle_pivots_equal_lapack_larger(orc, n, nb):
    A0 = orc.matgen(n, n, 100, kind=1)
    A = np.asfortranarray(A0.copy())
    ipiv, info = orc.pdgetrf(n, n, A, nb=nb)
    _, ipl, _ = orc.lapack_dgetrf(A0)
    np.testing.assert_array_equal(ipiv[:n], ipl)
    assert orc.fresid(A, ipiv[:n], A0) < 16


@pytest.mark.parametrize("nrhs", [1, 3, 9])
def test_oracle_solve_residual(orc, nrhs):
    n = 150
    A0 = orc.matgen(n, n, 100)
    B0 = orc.matgen(n, nrhs, 200)
    LU, ipiv, X, info = orc.solve_reference(A0, B0, nb=4)
    assert info == 0
    assert orc.sresid(A0, B0, X) < 1.0
    # LAPACK DGETRS on the same factors agrees
    Xl = np.asfortranarray(B0.copy())
    from oracle.oracle import lib, _p
    lib().orc_lapack_dgetrs(b"N", n, nrhs, _p(LU), n, _p(ipiv), _p(Xl), n)
    np.testing.assert_allclose(X, Xl, rtol=1e-10, atol=1e-12)


def test_oracle_transposed_solve(orc):
    n, nrhs = 97, 2
    A0 = orc.matgen(n, n, 100)
    B0 = orc.matgen(n, nrhs, 200)
    LU = np.asfortranarray(A0.copy())
    ipiv, info = orc.pdgetrf(n, n, LU, nb=8)
    X = np.asfortranarray(B0.copy())
    orc.pdgetrs("T", n, nrhs, LU, ipiv, X)
    assert orc.sresid(np.asfortranarray(A0.T), B0, X) < 1.0


def test_oracle_submatrix_offsets(orc):
    # sub(A) at (IA, JA) = (5, 5) inside a 20 x 20 array, NB = 4 (aligned)
    nb, ia, ja, n = 4, 5, 5, 12
    big = orc.matgen(20, 20, 100)
    A = np.asfortranarray(big.copy())
    ipiv = np.zeros(20 + nb, dtype=np.int32)
    ipiv, info = orc.pdgetrf(n, n, A, ia=ia, ja=ja, nb=nb, mglob=20, ipiv=ipiv)
    sub = np.asfortranarray(big[ia - 1:ia - 1 + n, ja - 1:ja - 1 + n].copy())
    ip2, info2 = orc.pdgetrf(n, n, sub, nb=nb)
    # IPIV(IA+k) holds global rows: IA + (relative pivot) - 1
    np.testing.assert_array_equal(ipiv[ia - 1:ia - 1 + n], ip2[:n] + ia - 1)
    np.testing.assert_array_equal(A[ia - 1:ia - 1 + n, ja - 1:ja - 1 + n], sub)
    # outside sub(A) untouched
    mask = np.ones_like(big, dtype=bool)
    mask[ia - 1:ia - 1 + n, ja - 1:ja - 1 + n] = False
    np.testing.assert_array_equal(A[mask], big[mask])


def test_oracle_singular_info(orc):
    n = 40
    A0 = orc.matgen(n, n, 100)
    A0[:, 7] = 0.0  # column 8 zero -> U(8,8) exactly zero
    A = np.asfortranarray(A0.copy())
    ipiv, info = orc.pdgetrf(n, n, A, nb=16)
    _, ipl, infol = orc.lapack_dgetrf(A0)
    assert info == infol == 8
    np.testing.assert_array_equal(ipiv[:n], ipl)


def test_plain_loop_blas_agrees_with_openblas(orc):
    n = 120
    A0 = orc.matgen(n, n, 100, kind=1)
    B0 = orc.matgen(n, 2, 200, kind=1)
    loaded = orc.blas_loaded()
    LU1, ip1, X1, _ = orc.solve_reference(A0, B0, nb=16)
    orc.use_fallback_blas()
    try:
        LU2, ip2, X2, _ = orc.solve_reference(A0, B0, nb=16)
    finally:
        if loaded:
            assert orc.reload_host_blas()
    np.testing.assert_array_equal(ip1, ip2)
    np.testing.assert_allclose(X1, X2, rtol=1e-10)


def test_near_tie_recorder_and_forced_replay(orc):
    n = 6
    A0 = orc.matgen(n, n, 100)
    A0[:, 0] = [0.5, 1.0, 1.0 + 1e-14, 0.3, -0.2, 0.1]  # rows 2 and 3 nearly tie
    rec = orc.Recorder(n)
    with rec:
        A = np.asfortranarray(A0.copy())
        ipiv, _ = orc.pdgetrf(n, n, A, nb=2)
    assert 0 in rec.near_ties()
    assert ipiv[0] == 3  # the larger of the two wins
    force = np.zeros(n, dtype=np.int32)
    force[0] = 2
    with orc.Recorder(n, force=force):
        A = np.asfortranarray(A0.copy())
        ipf, _ = orc.pdgetrf(n, n, A, nb=2)
    assert ipf[0] == 2


def test_conditioned_generator_singular_values(orc):
    n, kappa = 48, 1e4
    A = orc.gen_conditioned(n, kappa, nrefl=8, seed=1000)
    s = np.linalg.svd(A, compute_uv=False)
    np.testing.assert_allclose(s[0], 1.0, rtol=1e-10)
    np.testing.assert_allclose(s[0] / s[-1], kappa, rtol=1e-8)
