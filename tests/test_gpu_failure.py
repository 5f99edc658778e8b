"""Failure paths without a GPU fault: device-memory exhaustion is injected on
the host (sl1x1_debug_fail_alloc) at each growth of a library-owned buffer in
turn, after sl1x1_finalize has dropped them all. Every call must either
complete with a correct solution (the sliced-product scratch and the solve's
block inverses are optional: the FP64 DMMA update and the substitution solves
take over) or return INFO = -10002 (-10000 - cudaErrorMemoryAllocation); the
next call, with the hook off, must be correct again. No kernel is launched on
a missing buffer, so nothing here can fault the device.
"""
import numpy as np
import pytest

from lu_helpers import RESID_THRESH, system

pytestmark = pytest.mark.gpu
ENOMEM_INFO = -10002


@pytest.fixture(scope="module")
def ctx(sl, gpu_required):
    assert sl.lib().sl1x1_device_ok() == 1
    return sl.blacs_gridinit(1, 1)


def _pdgesv(sl, ctx, A0, B0, nb):
    n, nrhs = A0.shape[0], B0.shape[1]
    A = np.asfortranarray(A0.copy())
    X = np.asfortranarray(B0.copy())
    desca = np.array([1, ctx, n, n, nb, nb, 0, 0, n], np.int32)
    descb = np.array([1, ctx, n, nrhs, nb, nb, 0, 0, n], np.int32)
    ipiv = np.zeros(n + nb, np.int32)
    return sl.pdgesv(n, nrhs, A, 1, 1, desca, ipiv, X, 1, 1, descb), X


def test_pdgesv_exhaustion_at_each_growth(sl, orc, ctx):
    n, nrhs, nb = 600, 3, 64
    A0, B0 = system(orc, n, nrhs)
    L = sl.lib()
    failed = fell_back = 0
    try:
        for k in range(64):
            L.sl1x1_finalize()
            L.sl1x1_debug_fail_alloc(k)
            info, X = _pdgesv(sl, ctx, A0, B0, nb)
            fired = L.sl1x1_debug_fail_alloc(-1) < 0
            if not fired:
                assert info == 0
                break  # k is past the last growth of the call
            if info == 0:
                fell_back += 1
                assert orc.sresid(A0, B0, X) < RESID_THRESH
            else:
                assert info == ENOMEM_INFO
                failed += 1
            info, X = _pdgesv(sl, ctx, A0, B0, nb)
            assert info == 0
            assert orc.sresid(A0, B0, X) < RESID_THRESH
        else:
            pytest.fail("the hook still fired after 64 growths")
    finally:
        L.sl1x1_debug_fail_alloc(-1)
    assert failed >= 3 and fell_back >= 1, (failed, fell_back)


def test_mixed_exhaustion_at_each_growth(sl, orc, ctx):
    import torch

    n, nrhs = 1024, 1
    A0, B0 = system(orc, n, nrhs)
    L = sl.lib()
    dev = torch.device("cuda", 0)

    def run():
        dA = torch.from_numpy(np.ascontiguousarray(A0.T)).to(dev)
        dB = torch.from_numpy(np.ascontiguousarray(B0.T)).to(dev)
        dX = torch.zeros_like(dB)
        piv = torch.zeros(n, dtype=torch.int32, device=dev)
        info, _, _ = sl.dgesv_ir_dev(n, nrhs, dA.data_ptr(), n, piv.data_ptr(), dB.data_ptr(), n,
                                     dX.data_ptr(), n, fmt="bf16x3", nb=256)
        torch.cuda.synchronize()
        return info, np.asfortranarray(dX.cpu().numpy().T)

    failed = 0
    try:
        for k in range(64):
            L.sl1x1_finalize()
            L.sl1x1_debug_fail_alloc(k)
            info, X = run()
            fired = L.sl1x1_debug_fail_alloc(-1) < 0
            if not fired:
                assert info == 0
                break
            if info == 0:
                assert orc.sresid(A0, B0, X) < RESID_THRESH
            else:
                assert info == ENOMEM_INFO
                failed += 1
            info, X = run()
            assert info == 0
            assert orc.sresid(A0, B0, X) < RESID_THRESH
        else:
            pytest.fail("the hook still fired after 64 growths")
    finally:
        L.sl1x1_debug_fail_alloc(-1)
    assert failed >= 10, failed


@pytest.mark.parametrize("polls", [0, 1])
def test_panel_wait_runs_out_and_library_recovers(sl, orc, ctx, polls):
    """A device wait that gives up: with the panel's poll limit at 0 or 1, the
    cooperative panel's waits for the other CTAs' pivot candidates run out
    (no trap, no fault: each CTA records the timeout and returns, block 0
    writes identity pivots so the interchanges after it stay in range). The
    call returns INFO = -20002 (-20000 - kFlagTimeout); with the default
    limit restored the next call matches the oracle."""
    from lu_helpers import compare_ipiv

    n, nrhs, nb = 700, 2, 128  # 700 rows: six panel CTAs exchange candidates
    A0, B0 = system(orc, n, nrhs)
    L = sl.lib()
    try:
        L.sl1x1_debug_set_spin_limit(polls)
        info, X = _pdgesv(sl, ctx, A0, B0, nb)
        if polls == 0:
            assert info == -20002
        else:
            assert info in (-20002, 0)
    finally:
        L.sl1x1_debug_set_spin_limit(-1)
    A = np.asfortranarray(A0.copy())
    X = np.asfortranarray(B0.copy())
    desca = np.array([1, ctx, n, n, nb, nb, 0, 0, n], np.int32)
    descb = np.array([1, ctx, n, nrhs, nb, nb, 0, 0, n], np.int32)
    ipiv = np.zeros(n + nb, np.int32)
    assert sl.pdgesv(n, nrhs, A, 1, 1, desca, ipiv, X, 1, 1, descb) == 0
    bad, _ = compare_ipiv(orc, A0, ipiv[:n], nb)
    assert bad == 0
    assert orc.sresid(A0, B0, X) < RESID_THRESH
