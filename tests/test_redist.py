"""CPU tests of the block-cyclic redistribution (PDGEMR2D, REDIST/SRC/pdgemr.c):
the native per-pair pack / unpack against a numpy statement of the
block-cyclic mapping (every process pair of two layouts emulated in one
process), pdgemr2d_ on 1x1 contexts through the C ABI, and the cross-rank
form over torch.distributed with gloo ranks (world sizes 2 and 4)."""
import itertools
import os
import socket

import numpy as np
import pytest


def _layouts():
    from scalapack_gb300.redist import Layout

    return [
        (Layout(37, 23, 4, 3, 2, 3), Layout(37, 23, 5, 7, 3, 1, rsrc=1)),
        (Layout(10, 12, 2, 2, 1, 2, csrc=1), Layout(10, 12, 10, 12, 1, 1)),
        (Layout(64, 9, 8, 1, 4, 1), Layout(64, 9, 3, 2, 2, 2, rsrc=1, csrc=1)),
    ]


@pytest.mark.parametrize("case", range(3))
def test_pairwise_pack_unpack_matches_block_cyclic_map(sl, case):
    from scalapack_gb300 import redist as R

    la, lb = _layouts()[case]
    rng = np.random.default_rng(case)
    GA = rng.uniform(-1, 1, (la.m, la.n))
    GB = rng.uniform(-1, 1, (lb.m, lb.n))
    # a submatrix of A copied to a different place of B
    m, n = min(la.m, lb.m) - 3, min(la.n, lb.n) - 2
    ia, ja, ib, jb = 2, 3, 4, 1
    want = GB.copy()
    want[ib - 1:ib - 1 + m, jb - 1:jb - 1 + n] = GA[ia - 1:ia - 1 + m, ja - 1:ja - 1 + n]
    # every rank's local arrays (one grid rank = one list position)
    a_loc = {r: la.local_from_global(GA, r) for r in la.ranks}
    b_loc = {r: lb.local_from_global(GB, r) for r in lb.ranks}
    total = 0
    for sr, dr in itertools.product(la.ranks, lb.ranks):
        src, dst = la.coords(sr), lb.coords(dr)
        buf = R.pack(m, n, ia, ja, la, src, a_loc[sr], ib, jb, lb, dst)
        assert buf.size == R.pair_count(m, n, ia, ja, la, src, ib, jb, lb, dst)
        total += buf.size
        R.unpack(m, n, ia, ja, la, src, ib, jb, lb, dst, buf, b_loc[dr])
    assert total == m * n  # every element moves exactly once
    for r in lb.ranks:
        np.testing.assert_array_equal(b_loc[r], lb.local_from_global(want, r))


def test_pdgemr2d_abi_on_1x1_contexts(sl):
    ctx = sl.blacs_gridinit(1, 1)
    rng = np.random.default_rng(3)
    A = np.asfortranarray(rng.uniform(-1, 1, (30, 20)))
    B = np.asfortranarray(np.full((25, 40), -3.0))
    da = np.array([1, ctx, 30, 20, 4, 4, 0, 0, 30], np.int32)
    db = np.array([1, ctx, 24, 40, 8, 2, 0, 0, 25], np.int32)  # LLD 25 > M_B 24
    sl.pdgemr2d(12, 9, A, 5, 6, da, B, 3, 30, db, ctx)
    want = np.full((25, 40), -3.0)
    want[2:14, 29:38] = A[4:16, 5:14]
    np.testing.assert_array_equal(B, want)
    # out-of-bounds submatrix: nothing copied
    sl.pdgemr2d(12, 12, A, 5, 6, da, B, 3, 30, db, ctx)
    np.testing.assert_array_equal(B, want)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, grid, out_q):
    import torch.distributed as dist

    from scalapack_gb300.redist import Layout, pdgemr2d

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p, q = grid
        n, m = 45, 33
        rng = np.random.default_rng(99)
        G = rng.uniform(-1, 1, (m, n))
        la = Layout(m, n, 4, 5, p, q)
        root = Layout(m, n, 8, 8, 1, 1, ranks=[world - 1])  # gather to the last rank
        a_local = la.local_from_global(G, rank)
        full = np.zeros((m, n) if rank == world - 1 else (1, 1), order="F")
        pdgemr2d(m, n, a_local, 1, 1, la, full, 1, 1, root)
        ok_gather = (rank != world - 1) or bool(np.array_equal(full, G))
        # scatter a modified matrix back into the block-cyclic layout
        if rank == world - 1:
            full *= 2.0
        back = la.empty_local(rank)
        pdgemr2d(m, n, full, 1, 1, root, back, 1, 1, la)
        ok_scatter = bool(np.array_equal(back, la.local_from_global(2.0 * G, rank)))
        out_q.put((rank, ok_gather, ok_scatter))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("grid", [(1, 2), (2, 1), (2, 2)])
def test_pdgemr2d_across_gloo_ranks(sl, grid):
    import torch.multiprocessing as mp

    world = grid[0] * grid[1]
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    mp.start_processes(_worker, args=(world, _free_port(), grid, q), nprocs=world,
                       start_method="spawn", join=True)
    res = sorted(q.get() for _ in range(world))
    assert all(g and s for _, g, s in res), res
