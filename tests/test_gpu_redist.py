"""GPU test of the gather - solve - scatter PDGESV for a matrix distributed over
a 1x2 or 2x1 grid of gloo ranks: the root gathers sub(A) and sub(B) with
PDGEMR2D, factors and solves on the GPU, and every rank gets back its part of
L\\U, X and IPIV. Checked against the single-process pdgesv_ on the whole
matrix (identical factors, pivots and solution) and the oracle's residuals.
Only the root rank touches the GPU."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, grid, out_q):
    import torch.distributed as dist

    from scalapack_gb300.redist import Layout, pdgesv_gather

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        n, nrhs, nb = 300, 3, 32
        rng = np.random.default_rng(2024)
        A = rng.uniform(-0.5, 0.5, (n, n))
        B = rng.uniform(-0.5, 0.5, (n, nrhs))
        la = Layout(n, n, nb, nb, grid[0], grid[1])
        lb = Layout(n, nrhs, nb, nb, grid[0], grid[1])
        a_loc = la.local_from_global(A, rank)
        b_loc = lb.local_from_global(B, rank)
        pr, _ = la.coords(rank)
        ipiv = np.zeros(la.local_shape(*la.coords(rank))[0] + nb, np.int32)
        info = pdgesv_gather(n, nrhs, a_loc, la, ipiv, b_loc, lb, root=0)
        out_q.put((rank, info, a_loc, b_loc, ipiv, la.rows_of(pr), la.cols_of(la.coords(rank)[1]),
                   lb.cols_of(lb.coords(rank)[1])))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("grid", [(1, 2), (2, 1)])
def test_pdgesv_gather_matches_single_process(sl, orc, gpu_required, grid):
    import torch.multiprocessing as mp

    world = grid[0] * grid[1]
    ctxm = mp.get_context("spawn")
    q = ctxm.SimpleQueue()
    mp.start_processes(_worker, args=(world, _free_port(), grid, q), nprocs=world,
                       start_method="spawn", join=True)
    parts = [q.get() for _ in range(world)]
    n, nrhs, nb = 300, 3, 32
    rng = np.random.default_rng(2024)
    A = rng.uniform(-0.5, 0.5, (n, n))
    B = rng.uniform(-0.5, 0.5, (n, nrhs))
    # the same solve in this process through pdgesv_ directly
    ctx = sl.blacs_gridinit(1, 1)
    LU = np.asfortranarray(A.copy())
    X = np.asfortranarray(B.copy())
    ip = np.zeros(n + nb, np.int32)
    d = np.array([1, ctx, n, n, nb, nb, 0, 0, n], np.int32)
    db = np.array([1, ctx, n, nrhs, nb, nb, 0, 0, n], np.int32)
    assert sl.pdgesv(n, nrhs, LU, 1, 1, d, ip, X, 1, 1, db) == 0
    seen_rows = set()
    for rank, info, a_loc, b_loc, ipiv, rows, cols, bcols in parts:
        assert info == 0
        np.testing.assert_array_equal(a_loc[: len(rows), : len(cols)], LU[np.ix_(rows, cols)])
        np.testing.assert_array_equal(b_loc[: len(rows), : len(bcols)], X[np.ix_(rows, bcols)])
        np.testing.assert_array_equal(ipiv[: len(rows)], ip[rows])
        seen_rows |= set(rows.tolist())
    assert seen_rows == set(range(n))
    assert orc.sresid(np.asfortranarray(A), np.asfortranarray(B), X) < 16.0
