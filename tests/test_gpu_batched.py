"""GPU tests of the batched solver (plan -> CUDA-graph execution) through the
C ABI: every system's solution is checked against the CPU oracle's FP64 solve
with the tester's scaled residual, INFO is exact, inputs are untouched and a
second execution of the graph gives identical results."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_batch(rng, count, nmin=16, nmax=512, rmax=8, singular=None):
    systems = []
    for i in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        r = int(rng.integers(1, rmax + 1))
        A = np.asfortranarray(rng.uniform(-0.5, 0.5, size=(n, n)))
        if i % 2 == 0:
            A[np.diag_indices(n)] += n / 4.0  # diagonal shift on half the batch
        B = np.asfortranarray(rng.uniform(-0.5, 0.5, size=(n, r)))
        if singular is not None and i == singular:
            A[:, n // 3] = 0.0
        systems.append((A, B))
    return systems


class Plan:
    def __init__(self, sl, torch, systems, mode, autotune=1, tol=1.0):
        self.sl, self.torch = sl, torch
        self.dA = [torch.from_numpy(np.ascontiguousarray(A.T)).cuda() for A, _ in systems]
        self.dB = [torch.from_numpy(np.ascontiguousarray(B.T)).cuda() for _, B in systems]
        self.dX = [torch.zeros_like(b) for b in self.dB]
        k = len(systems)
        I = C.c_int * k
        P = C.c_void_p * k
        n = I(*[A.shape[0] for A, _ in systems])
        r = I(*[B.shape[1] for _, B in systems])
        self.batch = k
        self.plan = C.c_void_p()
        L = sl.lib()
        L.sl1x1_batch_plan_create.argtypes = [C.POINTER(C.c_void_p), C.c_int, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                              C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int,
                                              C.c_void_p]
        L.sl1x1_batch_plan_create.restype = C.c_int
        L.sl1x1_batch_plan_execute.argtypes = [C.c_void_p, C.c_void_p]
        L.sl1x1_batch_plan_results.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                               C.c_void_p]
        L.sl1x1_batch_plan_shape.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.sl1x1_batch_plan_destroy.argtypes = [C.c_void_p]
        torch.cuda.synchronize()
        info = L.sl1x1_batch_plan_create(
            C.byref(self.plan), k, n, r, P(*[t.data_ptr() for t in self.dA]), n,
            P(*[t.data_ptr() for t in self.dB]), n, P(*[t.data_ptr() for t in self.dX]), n, mode,
            tol, autotune, None)
        assert info == 0, info
        self.L = L

    def run(self):
        assert self.L.sl1x1_batch_plan_execute(self.plan, None) == 0
        info = (C.c_int * self.batch)()
        its = (C.c_int * self.batch)()
        sr = (C.c_double * self.batch)()
        assert self.L.sl1x1_batch_plan_results(self.plan, info, its, sr, None) == 0
        X = [np.asfortranarray(t.cpu().numpy().T) for t in self.dX]
        return list(info), list(its), list(sr), X

    def shape(self):
        t, c, s = C.c_int(), C.c_int(), C.c_int()
        self.L.sl1x1_batch_plan_shape(self.plan, C.byref(t), C.byref(c), C.byref(s))
        return t.value, c.value, s.value

    def close(self):
        self.L.sl1x1_batch_plan_destroy(self.plan)


@pytest.mark.parametrize("mode", [0, 1])
def test_batched_matches_oracle(sl, orc, gpu_required, mode):
    import torch

    rng = np.random.default_rng(100 + mode)
    systems = make_batch(rng, 48)
    plan = Plan(sl, torch, systems, mode)
    info, its, sr, X = plan.run()
    assert plan.shape()[0] in (128, 256, 512)
    for i, (A, B) in enumerate(systems):
        assert info[i] == 0
        r = orc.sresid(A, B, X[i])
        assert r < 16.0, (i, A.shape, r)
        # the kernel's own residual is at the same rounding-noise level (different summation order)
        assert sr[i] < 16.0 and sr[i] <= 10.0 * r + 0.1 and r <= 10.0 * sr[i] + 0.1, (sr[i], r)
        if mode == 1:
            assert its[i] >= 1 or its[i] == -1
    # inputs untouched
    for (A, B), dA, dB in zip(systems, plan.dA, plan.dB):
        np.testing.assert_array_equal(dA.cpu().numpy().T, A)
        np.testing.assert_array_equal(dB.cpu().numpy().T, B)
    # replaying the graph gives identical results
    info2, its2, sr2, X2 = plan.run()
    assert info2 == info and its2 == its
    for a, b in zip(X, X2):
        np.testing.assert_array_equal(a, b)
    plan.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_batched_singular_and_edges(sl, orc, gpu_required, mode):
    import torch

    rng = np.random.default_rng(7)
    systems = make_batch(rng, 9, nmin=1, nmax=70, rmax=8, singular=4)
    systems.append((np.asfortranarray(np.array([[2.0]])), np.asfortranarray(np.array([[3.0]]))))
    plan = Plan(sl, torch, systems, mode, autotune=0)
    info, its, sr, X = plan.run()
    A4 = systems[4][0]
    _, _, info_l = orc.lapack_dgetrf(A4)
    assert info[4] == info_l > 0
    for i, (A, B) in enumerate(systems):
        if i == 4:
            continue
        assert info[i] == 0
        assert orc.sresid(A, B, X[i]) < 16.0
    np.testing.assert_allclose(X[-1], [[1.5]])
    plan.close()


def test_batched_plan_rejects_bad_sizes(sl):
    L = sl.lib()
    saved = L.sl1x1_batch_plan_create.argtypes
    L.sl1x1_batch_plan_create.argtypes = None
    try:
        k = 1
        n = (C.c_int * k)(600)
        r = (C.c_int * k)(1)
        p = C.c_void_p()
        P = (C.c_void_p * k)(None)
        assert L.sl1x1_batch_plan_create(C.byref(p), k, n, r, P, n, P, n, P, n, 0, C.c_double(1.0),
                                         0, None) == -3
    finally:
        L.sl1x1_batch_plan_create.argtypes = saved
