"""sl1x1_dgetrf_noalloc: the FP64 factorization for callers that cannot
allocate GPU memory (a pool or arena that owns the device heap, a loop that may
not allocate after start-up). It keeps its scratch in a static 1 MiB device
array instead of library-owned buffers and runs the FP64 DMMA trailing update
(the sliced update's scratch grows with the matrix), so its results must be
exactly those of sl1x1_dgetrf_dev in that mode, call after call, even though
every call reuses the same scratch; against the default (sliced) entry point
the pivots are the same and the factors agree to rounding. This file is
collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest


def _factor_dev(sl, A0, nb, mode):
    """sl1x1_dgetrf_dev with the given trailing-update arithmetic."""
    sl.set_f64_update(mode)
    try:
        return _factor(sl, sl.dgetrf_dev, A0, nb)
    finally:
        sl.set_f64_update(1)


def _factor(sl, fn, A0, nb):
    import torch

    n = A0.shape[0]
    dA = torch.from_numpy(np.ascontiguousarray(A0.T)).cuda()  # column-major, ld = n
    dpiv = torch.zeros(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    info = fn(n, n, dA.data_ptr(), n, dpiv.data_ptr(), nb)
    return info, np.asfortranarray(dA.cpu().numpy().T), dpiv.cpu().numpy()


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point_twice(sl, gpu_required):
    rng = np.random.default_rng(7)
    n, nb = 900, 64
    A0 = np.asfortranarray(rng.uniform(-0.5, 0.5, size=(n, n)))
    info_r, LU_r, piv_r = _factor_dev(sl, A0, nb, 0)
    info_s, LU_s, piv_s = _factor_dev(sl, A0, nb, 1)
    assert info_r == info_s == 0
    for _ in range(2):  # two calls in a row share the static scratch
        info, LU, piv = _factor(sl, sl.dgetrf_noalloc, A0, nb)
        assert info == info_r
        np.testing.assert_array_equal(piv, piv_r)
        np.testing.assert_allclose(LU, LU_r, rtol=1e-12, atol=0)
        # the default entry point: same pivots, factors equal to rounding
        np.testing.assert_array_equal(piv, piv_s)
        assert np.max(np.abs(LU - LU_s)) < 1e-10


@pytest.mark.gpu
def test_noalloc_scratch_state_does_not_leak_between_calls(sl, gpu_required):
    rng = np.random.default_rng(8)
    n, nb = 300, 32
    S = np.asfortranarray(rng.uniform(-0.5, 0.5, size=(n, n)))
    S[:, 41] = 0.0  # exactly singular: INFO = 42
    R = np.asfortranarray(rng.uniform(-0.5, 0.5, size=(n, n)))
    assert _factor_dev(sl, S, nb, 1)[0] == 42
    assert _factor(sl, sl.dgetrf_noalloc, S, nb)[0] == 42
    info, LU, piv = _factor(sl, sl.dgetrf_noalloc, R, nb)  # the zero-pivot word was reset
    info_r, LU_r, piv_r = _factor_dev(sl, R, nb, 0)
    assert info == info_r == 0
    np.testing.assert_array_equal(piv, piv_r)
    np.testing.assert_allclose(LU, LU_r, rtol=1e-12, atol=0)


def test_noalloc_rejects_oversized_m_before_any_launch(sl, capfd):
    # Checked on the host before any device call, so it needs no GPU.
    info = sl.lib().sl1x1_dgetrf_noalloc(10 ** 6, 4, C.c_void_p(16), 10 ** 6, C.c_void_p(16), 64,
                                         None)
    assert info == -30000
    assert "exceeds the supported maximum" in capfd.readouterr().err


@pytest.mark.gpu
def test_noalloc_grows_no_library_buffer(sl, gpu_required):
    """The promise itself: with every library buffer dropped and the
    allocation-failure hook armed for the very next growth, the call
    completes and the hook never fires (nothing was allocated)."""
    rng = np.random.default_rng(9)
    n, nb = 400, 64
    A0 = np.asfortranarray(rng.uniform(-0.5, 0.5, size=(n, n)))
    info_r, LU_r, piv_r = _factor_dev(sl, A0, nb, 0)
    L = sl.lib()
    L.sl1x1_finalize()
    L.sl1x1_debug_fail_alloc(0)
    try:
        info, LU, piv = _factor(sl, sl.dgetrf_noalloc, A0, nb)
    finally:
        still_armed = L.sl1x1_debug_fail_alloc(-1)
    assert still_armed >= 0  # -1 would mean a library buffer grew
    assert info == info_r == 0
    np.testing.assert_array_equal(piv, piv_r)
    np.testing.assert_allclose(LU, LU_r, rtol=1e-12, atol=0)
