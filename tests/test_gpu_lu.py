"""GPU parity tests of the plain FP64 path through the C ABI (pdgesv_,
pdgetrf_, pdgetrs_ and the device entry points) against the CPU oracle.

Bar: IPIV identical to the oracle's except in logged near-tie columns (top-2
candidates within 1e-10 relative); scaled residuals ||A-PLU||/(||A|| max(M,N)
eps) and ||Ax-b||/(||A|| ||x|| N eps) below 16 (LIN/pdlafchk.f,
LIN/pdlaschk.f); exact INFO; untouched guard zones around every array.
"""
import json
import os

import numpy as np
import pytest

from lu_helpers import PADVAL, RESID_THRESH, compare_ipiv, guards_intact, padded, run_pdgesv, system

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
@pytest.fixture(scope="module")
def ctx(sl, gpu_required):
    assert sl.lib().sl1x1_device_ok() == 1
    return sl.blacs_gridinit(1, 1)


# NB 320 exceeds the composite row-interchange table (256 pivots) and takes the
# sequential interchange kernel for the outer swaps.
SMALL = [(1, 1), (2, 1), (3, 2), (31, 4), (64, 64), (65, 64), (257, 64), (257, 256), (1000, 64),
         (1000, 256), (513, 1), (100, 2), (700, 320)]


@pytest.mark.parametrize("n,nb", SMALL)
def test_pdgesv_small_parity(sl, orc, ctx, n, nb):
    A0, B0 = system(orc, n, 3)
    info, LU, rel, X = run_pdgesv(sl, ctx, A0, B0, nb)
    assert info == 0
    bad, ties = compare_ipiv(orc, A0, rel, nb)
    assert bad == 0, f"IPIV differs outside near-ties (ties logged: {ties})"
    assert orc.fresid(LU, rel, A0) < RESID_THRESH
    assert orc.sresid(A0, B0, X) < RESID_THRESH


def test_example_known_answer_gpu(sl, orc, ctx):
    d = json.load(open(os.path.join(GOLD, "dscaex.json")))
    n = d["n"]
    A0 = np.array(d["a_colmajor"]).reshape((n, n), order="F")
    B0 = np.array(d["b"]).reshape((n, 1), order="F")
    info, LU, rel, X = run_pdgesv(sl, ctx, A0, B0, d["nb"])
    assert info == 0
    np.testing.assert_allclose(X[:, 0], d["x_exact"], rtol=1e-13)
    assert orc.sresid(A0, B0, X) < d["threshold"]


@pytest.mark.parametrize("m,n", [(4, 4), (10, 12), (17, 13), (13, 13), (23, 23), (31, 31),
                                 (57, 50)])
@pytest.mark.parametrize("nb", [2, 3, 4, 5])
def test_pdgetrf_lu_dat_shapes(sl, orc, ctx, m, n, nb):
    # LU.dat sizes with the tester's own (-1,1] generator, factor only (M != N allowed)
    A0 = orc.matgen(m, n, 100, kind=0)
    Ab = padded(A0)
    desc = np.array([1, ctx, Ab.shape[0], Ab.shape[1], nb, nb, 0, 0, Ab.shape[0]], np.int32)
    ipiv = np.zeros(Ab.shape[0] + nb, dtype=np.int32)
    info = sl.pdgetrf(m, n, Ab, 1, 1, desc, ipiv)
    assert info == 0
    assert guards_intact(Ab, 1, 1, m, n)
    mn = min(m, n)
    LU = np.asfortranarray(Ab[:m, :n])
    bad, _ = compare_ipiv(orc, A0, ipiv[:mn], nb)
    assert bad == 0
    assert orc.fresid(LU, ipiv[:mn], A0) < 1.0  # LU.dat THRESH


def test_submatrix_offsets(sl, orc, ctx):
    nb, ia, ja, n = 8, 9, 17, 40
    A0, B0 = system(orc, n, 2)
    info, LU, rel, X = run_pdgesv(sl, ctx, A0, B0, nb, ia=ia, ja=ja)
    assert info == 0
    bad, _ = compare_ipiv(orc, A0, rel, nb)
    assert bad == 0
    assert orc.sresid(A0, B0, X) < RESID_THRESH


def test_singular_info_and_no_solve(sl, orc, ctx):
    n, nb = 80, 16
    A0, B0 = system(orc, n, 1)
    A0[:, 37] = 0.0
    info, LU, rel, X = run_pdgesv(sl, ctx, A0, B0, nb)
    _, _, infol = orc.lapack_dgetrf(A0)
    assert info == infol == 38
    np.testing.assert_array_equal(X, B0)  # PDGETRS skipped (pdgesv.f:231)
    bad, _ = compare_ipiv(orc, A0, rel, nb)
    assert bad == 0


def test_zero_matrix_info_one(sl, orc, ctx):
    n, nb = 10, 4
    A0 = np.zeros((n, n), order="F")
    Ab = padded(A0)
    desc = np.array([1, ctx, Ab.shape[0], Ab.shape[1], nb, nb, 0, 0, Ab.shape[0]], np.int32)
    ipiv = np.zeros(Ab.shape[0] + nb, dtype=np.int32)
    assert sl.pdgetrf(n, n, Ab, 1, 1, desc, ipiv) == 1
    np.testing.assert_array_equal(ipiv[:n], np.arange(1, n + 1))  # AMAX == 0 keeps the row


@pytest.mark.parametrize("trans", ["N", "T", "C"])
def test_pdgetrs_trans(sl, orc, ctx, trans):
    n, nb, nrhs = 300, 32, 5
    A0, B0 = system(orc, n, nrhs)
    A = np.asfortranarray(A0.copy())
    desc = np.array([1, ctx, n, n, nb, nb, 0, 0, n], np.int32)
    ipiv = np.zeros(n + nb, dtype=np.int32)
    assert sl.pdgetrf(n, n, A, 1, 1, desc, ipiv) == 0
    X = np.asfortranarray(B0.copy())
    descb = np.array([1, ctx, n, nrhs, nb, nb, 0, 0, n], np.int32)
    assert sl.pdgetrs(trans, n, nrhs, A, 1, 1, desc, ipiv, X, 1, 1, descb) == 0
    Aop = A0 if trans == "N" else np.asfortranarray(A0.T)
    assert orc.sresid(Aop, B0, X) < RESID_THRESH


def test_device_entry_points(sl, orc, ctx):
    import torch

    n, nrhs, nb = 777, 4, 64
    A0, B0 = system(orc, n, nrhs)
    ldda = 800
    dA = torch.zeros((n, ldda), dtype=torch.float64, device="cuda")  # column-major via transpose
    dA[:, :n] = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()
    dB = torch.from_numpy(np.ascontiguousarray(B0.T)).cuda()
    dpiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    info = sl.dgesv_dev(n, nrhs, dA.data_ptr(), ldda, dpiv.data_ptr(), dB.data_ptr(), n, nb)
    assert info == 0
    X = np.asfortranarray(dB.cpu().numpy().T)
    rel = dpiv.cpu().numpy()
    bad, _ = compare_ipiv(orc, A0, rel, nb)
    assert bad == 0
    assert orc.sresid(A0, B0, X) < RESID_THRESH


def test_config_n2048_nb64(sl, orc, ctx):
    # Plain FP64 PDGESV, N=2048, NB=64, NRHS=1, U[-0.5,0.5] from the seeded LCG
    n, nb = 2048, 64
    A0, B0 = system(orc, n, 1)
    info, LU, rel, X = run_pdgesv(sl, ctx, A0, B0, nb)
    assert info == 0
    bad, ties = compare_ipiv(orc, A0, rel, nb)
    assert bad == 0, ties
    assert orc.fresid(LU, rel, A0) < RESID_THRESH
    assert orc.sresid(A0, B0, X) < RESID_THRESH


@pytest.mark.parametrize("m,n,nb", [(2048, 2048, 64), (1000, 1000, 64), (3000, 3000, 256),
                                    (1500, 900, 64), (700, 1300, 64), (600, 600, 256)])
def test_host_path_chunked_copy_matches_device_path(sl, orc, ctx, m, n, nb):
    # pdgetrf_ / pdgesv_ copy A to the GPU in column chunks and run step 0 of
    # the factorization chunk by chunk as they land; the device entry points
    # get A whole. The interchanges and the trailing update are per column;
    # the U12 solve's first product balances its slices by the row maxima of
    # the columns it is given, so step 0's U12 rows agree to rounding rather
    # than bitwise. Pivots must be identical, factors and solution equal to
    # rounding.
    import torch

    rng = np.random.default_rng(m * 7 + n + nb)
    A0 = np.asfortranarray(rng.uniform(-0.5, 0.5, (m, n)))
    dA = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()
    mn = min(m, n)
    dpiv = torch.zeros(mn, dtype=torch.int32, device="cuda")
    assert sl.dgetrf_dev(m, n, dA.data_ptr(), m, dpiv.data_ptr(), nb) == 0
    LU_dev = np.asfortranarray(dA.cpu().numpy().T)
    piv_dev = dpiv.cpu().numpy()  # 1-based, as LAPACK's
    LU = np.asfortranarray(A0.copy())
    desca = np.array([1, ctx, m, n, nb, nb, 0, 0, m], np.int32)
    ipiv = np.zeros(m + nb, np.int32)
    assert sl.pdgetrf(m, n, LU, 1, 1, desca, ipiv) == 0
    np.testing.assert_array_equal(ipiv[:mn], piv_dev)
    scale = np.max(np.abs(LU_dev), axis=1, keepdims=True)
    assert np.max(np.abs(LU - LU_dev) / scale) < 1e-10
    if m == n:
        B0 = np.asfortranarray(rng.uniform(-0.5, 0.5, (n, 3)))
        dA = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()
        dB = torch.from_numpy(np.ascontiguousarray(B0.T)).cuda()
        assert sl.dgesv_dev(n, 3, dA.data_ptr(), n, dpiv.data_ptr(), dB.data_ptr(), n, nb) == 0
        X_dev = np.asfortranarray(dB.cpu().numpy().T)
        LU2, X = np.asfortranarray(A0.copy()), np.asfortranarray(B0.copy())
        descb = np.array([1, ctx, n, 3, nb, nb, 0, 0, n], np.int32)
        assert sl.pdgesv(n, 3, LU2, 1, 1, desca, ipiv, X, 1, 1, descb) == 0
        assert np.max(np.abs(LU2 - LU_dev) / scale) < 1e-10
        assert np.max(np.abs(X - X_dev)) <= 1e-10 * np.max(np.abs(X_dev))
        assert orc.sresid(A0, B0, X) < RESID_THRESH


@pytest.mark.parametrize("n,nb", [(3000, 256), (4096, 128)])
def test_update_sm_reserve_changes_no_bit(sl, orc, ctx, n, nb):
    # The look-ahead trailing update leaves SMs to the panel's stream by
    # capping its grid; each tile's product is the same whichever CTA computes
    # it, so the factors and pivots are bitwise those of the uncapped update.
    import torch

    L = sl.lib()
    rng = np.random.default_rng(n + nb)
    A0 = np.asfortranarray(rng.uniform(-0.5, 0.5, (n, n)))
    outs = []
    try:
        for lo, hi in ((0, 0), (24, 88), (120, 120), (8, 8)):
            L.sl1x1_set_update_reserve(lo, hi)
            dA = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()
            dpiv = torch.zeros(n, dtype=torch.int32, device="cuda")
            assert sl.dgetrf_dev(n, n, dA.data_ptr(), n, dpiv.data_ptr(), nb) == 0
            outs.append((dA.cpu().numpy(), dpiv.cpu().numpy()))
    finally:
        L.sl1x1_set_update_reserve(24, 88)
    for LU_t, piv in outs[1:]:
        np.testing.assert_array_equal(piv, outs[0][1])
        np.testing.assert_array_equal(LU_t, outs[0][0])
    assert orc.fresid(np.asfortranarray(outs[0][0].T), outs[0][1], A0) < RESID_THRESH


def test_config_n16384_nb256_full_size(sl, orc, ctx):
    # The headline case at full size: plain FP64 PDGESV, N=16384, NB=256,
    # NRHS=16, U[-0.5,0.5] from the tester's seeded generator. IPIV against
    # the oracle's pdgetrf (all host cores), then both scaled residuals.
    n, nb, nrhs = 16384, 256, 16
    orc.set_threads(os.cpu_count() or 1)
    A0, B0 = system(orc, n, nrhs)
    info, LU, rel, X = run_pdgesv(sl, ctx, A0, B0, nb)
    assert info == 0
    bad, ties = compare_ipiv(orc, A0, rel, nb)
    print(f"N={n}: {bad} pivot mismatches outside near ties; logged tie columns {ties}")
    assert bad == 0, ties
    assert orc.sresid(A0, B0, X) < RESID_THRESH
    assert orc.fresid(LU, rel, A0) < RESID_THRESH


@pytest.mark.parametrize("norm", ["M", "1", "O", "I", "F", "E"])
def test_pdlange_norms(sl, orc, ctx, norm):
    m, n = 300, 170
    A = orc.matgen(m, n, 100)
    Ab = padded(A, ia=5, ja=3)
    d = np.array([1, ctx, Ab.shape[0], Ab.shape[1], 4, 4, 0, 0, Ab.shape[0]], np.int32)
    v = sl.pdlange(norm, m, n, Ab, 5, 3, d)
    ref = {"M": np.abs(A).max(), "1": np.abs(A).sum(0).max(), "O": np.abs(A).sum(0).max(),
           "I": np.abs(A).sum(1).max(), "F": np.linalg.norm(A), "E": np.linalg.norm(A)}[norm]
    assert abs(v - ref) <= 1e-13 * ref


@pytest.mark.parametrize("norm", ["1", "I"])
@pytest.mark.parametrize("n", [2, 77, 600])
def test_pdgecon_brackets_true_rcond(sl, orc, ctx, norm, n):
    A0, _ = system(orc, n, 1)
    A = np.asfortranarray(A0.copy())
    nb = 32
    d = np.array([1, ctx, n, n, nb, nb, 0, 0, n], np.int32)
    ipiv = np.zeros(n + nb, dtype=np.int32)
    anorm = sl.pdlange(norm, n, n, A, 1, 1, d)
    assert sl.pdgetrf(n, n, A, 1, 1, d, ipiv) == 0
    rc, info, _, _ = sl.pdgecon(norm, n, A, 1, 1, d, anorm)
    assert info == 0
    inv = np.linalg.inv(A0)
    true = 1.0 / (anorm * (np.abs(inv).sum(0).max() if norm == "1" else np.abs(inv).sum(1).max()))
    # the estimate of ||inv(A)|| never exceeds the true norm, and is rarely far below it
    assert true * (1 - 1e-10) <= rc <= 10.0 * true, (rc, true)


@pytest.mark.parametrize("n,nb", [(1, 1), (5, 2), (200, 32), (1000, 64)])
def test_pdgetri_inverse(sl, orc, ctx, n, nb):
    A0, _ = system(orc, n, 1)
    A = np.asfortranarray(A0.copy())
    d = np.array([1, ctx, n, n, nb, nb, 0, 0, n], np.int32)
    ipiv = np.zeros(n + nb, dtype=np.int32)
    assert sl.pdgetrf(n, n, A, 1, 1, d, ipiv) == 0
    LU = np.asfortranarray(A.copy())
    info, _, _ = sl.pdgetri(n, A, 1, 1, d, ipiv)
    assert info == 0
    R = A0 @ A - np.eye(n)
    eps = 2.0 ** -53
    assert np.abs(R).sum(1).max() / (np.abs(A0).sum(1).max() * np.abs(A).sum(1).max() * n * eps) < 16
    # the oracle's restatement of the reference's algorithm on the same factors
    info_o, Xo = orc.pdgetri(LU, ipiv[:n] - 1, nb)
    assert info_o == 0
    assert np.abs(A - Xo).max() <= 1e-8 * np.abs(Xo).max()


def test_pdgetri_singular_info(sl, orc, ctx):
    n, nb = 50, 8
    A0, _ = system(orc, n, 1)
    A0[:, 20] = 0.0
    A = np.asfortranarray(A0.copy())
    d = np.array([1, ctx, n, n, nb, nb, 0, 0, n], np.int32)
    ipiv = np.zeros(n + nb, dtype=np.int32)
    k = sl.pdgetrf(n, n, A, 1, 1, d, ipiv)
    assert k == 21
    before = A.copy()
    info, _, _ = sl.pdgetri(n, A, 1, 1, d, ipiv)
    assert info == 21
    np.testing.assert_array_equal(A, before)  # inverse not computed


def test_tall_matrix_beyond_shared_memory_panel(sl, orc, ctx):
    """M = 200,000 > 152 SMs x 768 rows: the panel's rows no longer fit the
    SMs' shared memory, and each CTA keeps its rows in a library-owned global
    buffer instead. pdgetrf_ on a 200000 x 512 matrix (0.8 GB): IPIV identical
    to the oracle's, the tester's factor residual below 16."""
    m, n, nb = 200000, 512, 256
    assert m > 152 * 768
    A0 = orc.matgen(m, n, 100, kind=1)
    A = np.asfortranarray(A0.copy())
    desc = np.array([1, ctx, m, n, nb, nb, 0, 0, m], np.int32)
    ipiv = np.zeros(m + nb, np.int32)
    assert sl.pdgetrf(m, n, A, 1, 1, desc, ipiv) == 0
    bad, ties = compare_ipiv(orc, A0, ipiv[:n], nb)
    assert bad == 0, ties
    assert orc.fresid(A, ipiv[:n], A0) < RESID_THRESH


@pytest.mark.parametrize("n,nb", [(200, 32), (1000, 64)])
def test_scratch_on_reused_dirty_memory(sl, orc, ctx, n, nb):
    # The sliced products keep epoch-tagged balancing words at the start of
    # their scratch buffers; a buffer allocated over memory that held other
    # data (here: all bits set, freed back to the driver) must start clean,
    # or the words of later products would never replace the stale ones.
    import torch

    L = sl.lib()
    L.sl1x1_finalize()
    junk = torch.full((1 << 27,), -1, dtype=torch.int64, device="cuda")  # 1 GiB of 0xff
    torch.cuda.synchronize()
    del junk
    torch.cuda.empty_cache()
    rng = np.random.default_rng(n + 3)
    A0 = np.asfortranarray(rng.uniform(-1, 1, (n, n)))
    dA = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()
    dpiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    assert sl.dgetrf_dev(n, n, dA.data_ptr(), n, dpiv.data_ptr(), nb) == 0
    LU = np.asfortranarray(dA.cpu().numpy().T)
    assert orc.fresid(LU, dpiv.cpu().numpy(), A0) < RESID_THRESH
