"""CPU models of the index logic in three GPU routines, checked against the
plain sequential definitions they replace:

* factor_panel's in-panel blocks (lu_f64.cu): 32-column sub-panels grouped in
  blocks of IB; after each sub-panel only the next sub-panel's columns are
  brought up to date (a strip solve over the block's pivot rows so far and a
  product with k = those rows), and at the end of a block every remaining
  column (k = the block's rows). Any IB must give the pivots of the plain
  right-looking order (IB = 1) and factors equal to rounding.
* perm_compose_kernel (lu_f64.cu): perm[i], the original row that ends in row
  i after the interchanges j <-> ipiv[j], by a backward walk per row.
* laswp_plan_block (lu_kernels.cuh): the (row, src) pairs of a panel's
  interchanges by a backward walk per touched row, in the order a sequential
  replay produces them.
"""
import numpy as np
import pytest

PW = 32


def _factor_panel(A, ipiv, j, jb, ib):
    m = A.shape[0]
    blk_r0 = j
    c, q = 0, 0
    while c < jb:
        w = min(PW, jb - c)
        r0 = j + c
        kw = min(m - r0, w)
        # the cooperative sub-panel kernel: PDGETF2 on rows r0.., columns r0..r0+w
        for k in range(kw):
            col = r0 + k
            p = r0 + k + int(np.argmax(np.abs(A[r0 + k:, col])))
            ipiv[col] = p
            if p != col:
                A[[col, p], r0:r0 + w] = A[[p, col], r0:r0 + w]
            A[col + 1:, col] /= A[col, col]
            A[col + 1:, col + 1:r0 + w] -= np.outer(A[col + 1:, col], A[col, col + 1:r0 + w])
        # its interchanges on the panel's other columns
        for k in range(kw):
            col = r0 + k
            p = ipiv[col]
            if p != col:
                for cs in (slice(j, r0), slice(r0 + w, j + jb)):
                    A[[col, p], cs] = A[[p, col], cs]
        if c + w < jb:
            block_end = (q + 1) % ib == 0 or kw < w
            ncols = jb - c - w if block_end else min(jb - c - w, PW)
            kb = r0 + kw - blk_r0
            rl = r0 + kw
            lt = np.tril(A[blk_r0:blk_r0 + kb, blk_r0:blk_r0 + kb], -1) + np.eye(kb)
            cols = slice(r0 + w, r0 + w + ncols)
            A[blk_r0:blk_r0 + kb, cols] = np.linalg.solve(lt, A[blk_r0:blk_r0 + kb, cols])
            if rl < m:
                A[rl:, cols] -= A[rl:, blk_r0:blk_r0 + kb] @ A[blk_r0:blk_r0 + kb, cols]
            if block_end:
                blk_r0 = r0 + w
        c += PW
        q += 1


def _lu(A0, nb, ib):
    A = A0.copy()
    m, n = A.shape
    mn = min(m, n)
    ipiv = np.zeros(mn, int)
    for j in range(0, mn, nb):
        jb = min(nb, mn - j)
        _factor_panel(A, ipiv, j, jb, ib)
        for k in range(j, j + jb):
            p = ipiv[k]
            if p != k:
                A[[k, p], :j] = A[[p, k], :j]
                A[[k, p], j + jb:] = A[[p, k], j + jb:]
        if j + jb < n:
            lt = np.tril(A[j:j + jb, j:j + jb], -1) + np.eye(jb)
            A[j:j + jb, j + jb:] = np.linalg.solve(lt, A[j:j + jb, j + jb:])
            A[j + jb:, j + jb:] -= A[j + jb:, j:j + jb] @ A[j:j + jb, j + jb:]
    return A, ipiv


@pytest.mark.parametrize("m,n,nb", [(300, 300, 256), (257, 257, 96), (200, 200, 48),
                                    (130, 90, 256), (90, 130, 64), (70, 70, 33)])
@pytest.mark.parametrize("ib", [2, 3, 4, 8])
def test_in_panel_blocks_keep_the_pivots(m, n, nb, ib):
    rng = np.random.default_rng(m * 3 + n + nb)
    A0 = rng.uniform(-1, 1, (m, n))
    ref, rp = _lu(A0, nb, 1)
    lu, p = _lu(A0, nb, ib)
    np.testing.assert_array_equal(p, rp)
    assert np.abs(lu - ref).max() < 1e-11 * max(1.0, np.abs(ref).max())
    # and it is an LU of A: P A = L U
    mn = min(m, n)
    L = np.tril(lu[:, :mn], -1) + np.eye(m, mn)
    U = np.triu(lu[:mn, :])
    PA = A0.copy()
    for i in range(mn):
        if p[i] != i:
            PA[[i, p[i]]] = PA[[p[i], i]]
    assert np.abs(PA - L @ U).max() < 1e-11 * m


def _perm_walk(ipiv):
    n = len(ipiv)
    out = np.empty(n, int)
    for i in range(n):
        q = i
        for j in range(n - 1, -1, -1):
            p = ipiv[j]
            q = p if q == j else (j if q == p else q)
        out[i] = q
    return out


def test_permutation_walk_matches_sequential_interchanges():
    rng = np.random.default_rng(11)
    for trial in range(200):
        n = int(rng.integers(1, 50))
        # LAPACK pivots (ipiv[j] >= j) and arbitrary in-range ones
        ipiv = ([int(rng.integers(j, n)) for j in range(n)] if trial % 2
                else [int(v) for v in rng.integers(0, n, size=n)])
        p = list(range(n))
        for i in range(n):
            q = ipiv[i]
            p[i], p[q] = p[q], p[i]
        np.testing.assert_array_equal(_perm_walk(ipiv), p)


def _plan_replay(k1, k2, piv):
    row = list(range(k1, k2))
    src = list(range(k1, k2))
    tab = {}
    for i in range(k2 - k1):
        p = piv[i]
        if p == k1 + i:
            continue
        if k1 <= p < k2:
            e = p - k1
        else:
            if p not in tab:
                tab[p] = len(row)
                row.append(p)
                src.append(p)
            e = tab[p]
        src[i], src[e] = src[e], src[i]
    return [(r, s) for r, s in zip(row, src) if r != s]


def _plan_walk(k1, k2, piv):
    npiv = k2 - k1
    first = [(p < k1 or p >= k2) and all(piv[i2] != p for i2 in range(i)) for i, p in enumerate(piv)]
    rows = list(range(k1, k2)) + [p for i, p in enumerate(piv) if first[i]]
    out = []
    for r in rows:
        q = r
        for i in range(npiv - 1, -1, -1):
            p = piv[i]
            q = p if q == k1 + i else (k1 + i if q == p else q)
        if q != r:
            out.append((r, q))
    return out


def test_interchange_plan_walk_matches_replay():
    rng = np.random.default_rng(3)
    for _ in range(300):
        k1 = int(rng.integers(0, 50))
        npiv = int(rng.integers(1, 40))
        m = k1 + npiv + int(rng.integers(0, 60))
        piv = [int(rng.integers(k1 + i, m)) for i in range(npiv)]
        assert _plan_walk(k1, k1 + npiv, piv) == _plan_replay(k1, k1 + npiv, piv)
